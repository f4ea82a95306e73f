// sg_raster.cuh -- rasterization, pixel shading and output merging of a pass.
//
// Three kernels per pass after binning:
//   k_cover   work items are squares of a tile (its four 32x32 quadrants,
//             or sixteen 16x16 regions for crowded tiles), dynamically
//             scheduled over every tile of every target; 128 threads.  Each
//             owned 4x4 block replays, in primitive order, the reference's
//             64 -> 16 -> 4 -> sample classification, quad coverage and
//             early-Z.  Surviving quads become fragments in per-owner lists
//             (an owner per 2x2 quad of the tile; this kernel fills the list
//             of each block's top-left quad).  sg_cover.cu's k_cover2 is the
//             default coverage kernel.
//   k_shade   every fragment of the pass, 4 lanes per quad (one per pixel):
//             attribute interpolation and the pixel-shader program, with
//             ddx/ddy from the quad's lanes.  One instance per varying count
//             (and learned-filter instances), walking the fragment lists
//             k_frag_classes groups by shade class and program.
//   k_merge   warps take 32 owners of a tile at a time from a device-wide
//             cursor; each owner walks its fragments in primitive order and
//             applies depth-stencil (when early-Z is off) and the blend
//             program per covered sample.
// Included by sg_raster_a.cu / _b.cu / _c.cu, which instantiate k_shade for
// two varying counts each so the translation units compile in parallel.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "sg_draw.cuh"
#include "sg_learned.cuh"

namespace sg {

struct TriView {
  float4 const* R;
  int nreg;
  __device__ float4 edge(int i) const { return R[i]; }
  __device__ float4 bbox() const { return R[3]; }
  __device__ bool front() const { return (rec_flag_bits(R) >> 31) != 0u; }
  __device__ v4 v0(int i) const { return ld4(R + 5 + i); }
  __device__ v4 ddx(int i) const { return ld4(R + 5 + nreg + i); }
  __device__ v4 ddy(int i) const { return ld4(R + 5 + 2 * nreg + i); }
};

// Compare functions: SG_CMP_* are the reference's values (LESS 1, EQUAL 2,
// GREATER 4 and their unions), so a function passes when the bit of the
// operands' ordering is set.  Unordered float operands (NaN) pass NOT_EQUAL
// and ALWAYS only, as `a != b` and `true` do; values above ALWAYS pass.
// Branch-free: the function is data, and a switch per sample diverges.
__device__ inline bool cmpf(uint32_t f, float a, float b) {
  bool const lt = a < b, eq = a == b, gt = a > b;
  return ((f & 1u) && lt) || ((f & 2u) && eq) || ((f & 4u) && gt) || ((f & 5u) == 5u && !(lt || eq || gt)) || f > 7u;
}
__device__ inline bool cmpu(uint32_t f, uint32_t a, uint32_t b) {
  return ((f & 1u) && a < b) || ((f & 2u) && a == b) || ((f & 4u) && a > b) || f > 7u;
}
__device__ inline uint32_t stencil_op(uint32_t op, uint32_t ref, uint32_t cur) {  // framebuffer.cpp:136-166
  switch (op) {
  case SG_SOP_KEEP: return cur;
  case SG_SOP_ZERO: return 0;
  case SG_SOP_REPLACE: return ref;
  case SG_SOP_INCR_SAT: return min(0xFFu, cur + 1);
  case SG_SOP_DECR_SAT: return cur - 1;  // std::max<uint32_t>(0, cur - 1) keeps the wrapped value
  case SG_SOP_INVERT: return ~cur;
  case SG_SOP_INCR_WRAP: return (cur + 1) & 0xFF;
  case SG_SOP_DECR_WRAP: return (cur - 1 + 256) & 0xFF;
  default: return cur;
  }
}
// EXTENSION (D24S8): depth quantised to 24-bit unorm, round to nearest even
__device__ inline uint32_t d24_quantize(float z) {
  float c = fminf(fmaxf(z, 0.0f), 1.0f) * 16777215.0f;
  return __float2uint_rn(c);
}

struct DSVal {
  float depth;
  uint32_t q;
  uint32_t stencil;
};

__device__ inline DSVal ds_read(TargetParams const& T, DrawParams const& D, uint8_t const* a) {
  DSVal v{0.0f, 0u, 0u};
  switch (T.ds_fmt) {
  case SG_FMT_RG32F:
    if (D.read_depth) v.depth = *reinterpret_cast<float const*>(a);
    if (D.stencil) v.stencil = reinterpret_cast<uint32_t const*>(a)[1] & D.read_mask;
    break;
  case SG_FMT_D32F:
    if (D.read_depth) v.depth = *reinterpret_cast<float const*>(a);
    break;
  case SG_FMT_D24S8: {
    uint32_t w = *reinterpret_cast<uint32_t const*>(a);
    if (D.read_depth) v.q = w & 0xFFFFFFu;
    if (D.stencil) v.stencil = (w >> 24) & D.read_mask;
    break;
  }
  default: break;
  }
  return v;
}
__device__ inline void ds_write(TargetParams const& T, DrawParams const& D, uint8_t* a, float depth,
                                uint32_t stencil, uint32_t wmask) {
  switch (T.ds_fmt) {
  case SG_FMT_RG32F:
    if (D.write_depth) *reinterpret_cast<float*>(a) = depth;
    if (D.stencil) reinterpret_cast<uint32_t*>(a)[1] = stencil & wmask;
    break;
  case SG_FMT_D32F:
    if (D.write_depth) *reinterpret_cast<float*>(a) = depth;
    break;
  case SG_FMT_D24S8: {
    uint32_t w = *reinterpret_cast<uint32_t*>(a);
    if (D.write_depth) w = (w & 0xFF000000u) | d24_quantize(depth);
    if (D.stencil) w = (w & 0x00FFFFFFu) | ((stencil & wmask & 0xFFu) << 24);
    *reinterpret_cast<uint32_t*>(a) = w;
    break;
  }
  default: break;
  }
}
__device__ inline bool depth_pass(TargetParams const& T, DrawParams const& D, float depth, DSVal const& old) {
  if (T.ds_fmt == SG_FMT_D24S8 && D.read_depth) return cmpu(D.depth_func, d24_quantize(depth), old.q);
  return cmpf(D.depth_func, depth, old.depth);
}
__device__ inline uint8_t* ds_addr(TargetParams const& T, uint32_t x, uint32_t y, uint32_t s) {
  return T.ds + ((static_cast<size_t>(y) * T.ds_width + x) * T.samples + s) * T.ds_esz;
}
__device__ inline uint8_t* color_addr(TargetParams const& T, uint32_t x, uint32_t y, uint32_t s) {
  return T.color + ((static_cast<size_t>(y) * T.color_stride + x) * T.samples + s) * T.color_esz;
}

// cpp_blend_shader programs; `more` holds the pixel's colours 1.. (or null)
__device__ inline void blend(TargetParams const& T, DrawParams const& D, uint32_t x, uint32_t y, uint32_t s, v4 src,
                             float4 const* more) {
  if (!T.color) return;
  uint8_t* a = color_addr(T, x, y, s);
  if (D.bs_prog == SG_BS_REPLACE_ALL) {  // color(i, s) = in.color[i] for every bound target
    write_texel(T.color_fmt, a, src);
    for (uint32_t i = 0; i < T.nmore; ++i) {
      float4 const c = more ? more[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      write_texel(T.more_fmt[i],
                  T.more_color[i] + ((static_cast<size_t>(y) * T.more_stride[i] + x) * T.samples + s) * T.more_esz[i],
                  mk4(c.x, c.y, c.z, c.w));
    }
    return;
  }
  switch (D.bs_prog) {
  case SG_BS_LERP_SRC_ALPHA: {
    v4 d = read_texel(T.color_fmt, a);
    write_texel(T.color_fmt, a, mk4(lerp1(d.x, src.x, src.w), lerp1(d.y, src.y, src.w), lerp1(d.z, src.z, src.w),
                                    lerp1(d.w, src.w, src.w)));
    break;
  }
  case SG_BS_ADD: write_texel(T.color_fmt, a, read_texel(T.color_fmt, a) + src); break;
  default: write_texel(T.color_fmt, a, src); break;
  }
}

// The 4-byte colour formats as words (read_texel / write_texel, the same
// conversions), and the blend programs on a decoded value.
__device__ inline v4 decode_word(uint32_t fmt, uint32_t u) {
  switch (fmt) {
  case SG_FMT_BGRA8: return unorm8_word_to_f(u, false);
  case SG_FMT_RGBA8: return unorm8_word_to_f(u, true);
  case SG_FMT_R32F: return mk4(__uint_as_float(u), 0.0f, 0.0f, 0.0f);
  case SG_FMT_R32I: return mk4(static_cast<float>(static_cast<int32_t>(u)), 0.0f, 0.0f, 0.0f);
  default: return mk4(0, 0, 0, 0);
  }
}
__device__ inline uint32_t encode_word(uint32_t fmt, v4 c) {
  switch (fmt) {
  case SG_FMT_BGRA8: return f_to_unorm8(c.z) | (f_to_unorm8(c.y) << 8) | (f_to_unorm8(c.x) << 16) | (f_to_unorm8(c.w) << 24);
  case SG_FMT_RGBA8: return f_to_unorm8(c.x) | (f_to_unorm8(c.y) << 8) | (f_to_unorm8(c.z) << 16) | (f_to_unorm8(c.w) << 24);
  case SG_FMT_R32F: return __float_as_uint(c.x);
  case SG_FMT_R32I: return static_cast<uint32_t>(static_cast<int32_t>(c.x + 0.5f));
  default: return 0u;
  }
}
__device__ inline uint32_t blend_word(uint32_t fmt, uint32_t bs_prog, uint32_t dst, v4 src) {
  switch (bs_prog) {
  case SG_BS_LERP_SRC_ALPHA: {
    v4 d = decode_word(fmt, dst);
    return encode_word(fmt, mk4(lerp1(d.x, src.x, src.w), lerp1(d.y, src.y, src.w), lerp1(d.z, src.z, src.w),
                                lerp1(d.w, src.w, src.w)));
  }
  case SG_BS_ADD: return encode_word(fmt, decode_word(fmt, dst) + src);
  default: return encode_word(fmt, src);
  }
}

// A user blend shader's body on one sample (defined with the user shader
// kernels, sg_user.cuh).
template <class UBS>
__device__ void user_blend(TargetParams const& T, DrawParams const& D, uint32_t x, uint32_t y, uint32_t s, v4 src,
                           float4 const* more);
// The draw's blend program: a stock one, or UBS's body for a user program.
template <class UBS>
__device__ inline void blend_t(TargetParams const& T, DrawParams const& D, uint32_t x, uint32_t y, uint32_t s, v4 src,
                               float4 const* more) {
  if constexpr (!std::is_void<UBS>::value) {
    if (D.bs_prog >= SG_USER_PROGRAM_BASE) {
      user_blend<UBS>(T, D, x, y, s, src, more);
      return;
    }
  }
  blend(T, D, x, y, s, src, more);
}

// framebuffer::render_sample (framebuffer.cpp:445-479)
template <class UBS = void>
__device__ inline void render_sample(TargetParams const& T, DrawParams const& D, uint32_t x, uint32_t y, uint32_t s,
                                     v4 src, float depth, bool front, float4 const* more) {
  if (D.early_z || !T.ds) {
    blend_t<UBS>(T, D, x, y, s, src, more);
    return;
  }
  uint8_t* a = ds_addr(T, x, y, s);
  DSVal old = ds_read(T, D, a);
  bool dp = depth_pass(T, D, depth, old);
  uint32_t func = front ? D.front_func : D.back_func;
  bool sp = D.stencil ? cmpu(func, D.stencil_ref, old.stencil) : true;
  if (dp && sp) {
    uint32_t ns = D.stencil ? stencil_op(front ? D.front_pass : D.back_pass, D.stencil_ref, old.stencil) : 0u;
    blend_t<UBS>(T, D, x, y, s, src, more);
    ds_write(T, D, a, depth, ns, D.write_mask);
  }
}

// Coverage-pass copy of a triangle in shared memory: what coverage and early-Z
// read (edges, bounding box, the position register of v0 / ddx / ddy), and
// the draw's early-Z configuration and shade key.
struct TriStage {
  float4 bbox, e0, e1, e2, p0, dpx, dpy;
  uint32_t entry, zcfg, shade_key, pad;
};
struct StageView {
  TriStage const* S;
  __device__ float4 edge(int i) const { return i == 0 ? S->e0 : i == 1 ? S->e1 : S->e2; }
  __device__ float4 bbox() const { return S->bbox; }
  __device__ v4 v0(int) const { return mk4(S->p0.x, S->p0.y, S->p0.z, S->p0.w); }
  __device__ v4 ddx(int) const { return mk4(S->dpx.x, S->dpx.y, S->dpx.z, S->dpx.w); }
  __device__ v4 ddy(int) const { return mk4(S->dpy.x, S->dpy.y, S->dpy.z, S->dpy.w); }
};

// step_2d_unproj_pos_quad, one pixel of the quad (shader.cpp:257-287)
template <class TV>
__device__ inline v4 quad_pos(TV const& t, float dx, float dy, int q) {
  v4 in = t.v0(0), d0 = t.ddx(0), d1 = t.ddy(0);
  v4 p00 = mk4(in.x + (d0.x * dx + d1.x * dy), in.y + (d0.y * dx + d1.y * dy), in.z + (d0.z * dx + d1.z * dy),
               in.w + (d0.w * dx + d1.w * dy));
  if (q == 0) return p00;
  if (q == 1) return p00 + d0;
  if (q == 2) return p00 + d1;
  return (p00 + d0) + d1;
}

// 64-bit quad mask (16 bits per pixel, <= 4 samples used) <-> 16-bit compact form
__device__ inline uint32_t compact_mask(uint64_t m) {
  return static_cast<uint32_t>((m & 0xF) | ((m >> 12) & 0xF0) | ((m >> 24) & 0xF00) | ((m >> 36) & 0xF000));
}
__device__ inline uint64_t expand_mask(uint32_t c) {
  return static_cast<uint64_t>(c & 0xF) | (static_cast<uint64_t>((c >> 4) & 0xF) << 16) |
         (static_cast<uint64_t>((c >> 8) & 0xF) << 32) | (static_cast<uint64_t>((c >> 12) & 0xF) << 48);
}

// An owner's append cursor into its chunked fragment list.
struct OwnerList {
  uint32_t first, cur, count;  // first chunk, current chunk, slots used in it
};

__device__ inline bool owner_append(PassParams const& P, OwnerList& L, uint32_t rec, uint32_t pos, uint32_t mask) {
  // a new chunk when the list has none or its chunk is full: the threads of
  // the warp appending together take theirs with one atomic on the shared
  // counter (one address every SM allocates from)
  bool const need = L.cur == NO_CHUNK || L.count == FRAG_CHUNK;
  unsigned const act = __activemask();
  unsigned const want = __ballot_sync(act, need);
  if (need) {
    unsigned const lane = threadIdx.x & 31u;
    int const leader = __ffs(want) - 1;
    uint32_t base = 0;
    if (static_cast<int>(lane) == leader) base = atomicAdd(&P.counters->chunk_total, static_cast<uint32_t>(__popc(want)));
    base = __shfl_sync(want, base, leader);
    uint32_t const c = base + static_cast<uint32_t>(__popc(want & ((1u << lane) - 1u)));
    if (c >= P.chunk_capacity) {
      atomicOr(&P.counters->overflow, OVF_FRAG);
      return false;
    }
    if (L.cur == NO_CHUNK) {
      L.first = c;
    } else {
      P.chunk_next[L.cur] = c;
      P.chunk_count[L.cur] = FRAG_CHUNK;
    }
    L.cur = c;
    L.count = 0;
  }
  uint32_t f = L.cur * FRAG_CHUNK + L.count++;
  P.frag_rec[f] = rec;
  P.frag_pos[f] = pos;
  P.frag_mask[f] = mask;
  return true;
}

// Per-level edge parameters of one triangle: TILE * e, then * 0.25 per level
// (rasterizer.cpp:668-710).
struct LevelParams {
  float stx[3], sty[3], r2a[3], ev[3];
};
__device__ inline void level_params(float4 const* e, LevelParams& l1, LevelParams& l2) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    bool mx = e[k].x > 0, my = e[k].y > 0;
    float stx = TILE * e[k].x, sty = TILE * e[k].y;
    float r2a = -fabsf(stx) - fabsf(sty);
    float pev = static_cast<float>(mx * TILE) * e[k].x + static_cast<float>(my * TILE) * e[k].y;
    stx *= 0.25f; sty *= 0.25f; r2a *= 0.25f; pev *= 0.25f;
    l1.stx[k] = stx; l1.sty[k] = sty; l1.r2a[k] = r2a; l1.ev[k] = e[k].z - pev;
    stx *= 0.25f; sty *= 0.25f; r2a *= 0.25f; pev *= 0.25f;
    l2.stx[k] = stx; l2.sty[k] = sty; l2.r2a[k] = r2a; l2.ev[k] = e[k].z - pev;
  }
}

// subdivide_tile's trivial reject / accept of child (ix, iy) of the region at
// (left, top) (rasterizer.cpp:485-540): 0 = rejected, 1 = partial, 2 = accepted.
__device__ inline int child_class(float4 const* e, LevelParams const& l, float left, float top, int ix, int iy) {
  bool rej = false, accf = false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float ev3 = l.ev[k] - (left * e[k].x + top * e[k].y);
    float srej = l.stx[k] * static_cast<float>(ix) + l.sty[k] * static_cast<float>(iy);
    rej = rej || (srej < ev3);
    accf = accf || ((srej + l.r2a[k]) < ev3);
  }
  return rej ? 0 : (accf ? 1 : 2);
}

__device__ inline uint32_t target_of_tile(PassParams const& P, uint32_t tile) {
  return upper_index(P.target_tile_base, P.ntargets, tile);
}

#ifdef SG_RASTER_COVER_MERGE  // defined by the one translation unit that owns these kernels
constexpr int STAGE_TRIS = 256;  // triangles staged in shared memory per batch
constexpr int MASK_WORDS = STAGE_TRIS / 32;
constexpr int COVER_THREADS = 128;  // one CTA per 32x32 quadrant of a tile
constexpr int QUAD_PX = 32;
constexpr size_t COVER_SMEM_BASE = STAGE_TRIS * sizeof(TriStage) + (64 + 4) * MASK_WORDS * sizeof(uint32_t);
// plus the staged depth: QUAD_PX * QUAD_PX * samples words (only when early-Z is on)
__host__ __device__ constexpr size_t cover_smem(uint32_t samples, bool early_z) {
  return COVER_SMEM_BASE + (early_z ? static_cast<size_t>(QUAD_PX) * QUAD_PX * samples * 4 : 0);
}

// The sample slots a lane covers in a (triangle, block) pair: slot lane + 32
// pass of the block's 16 pixels x samples, pixel-major.  Fixed per target.
struct LaneSlots {
  uint32_t bit[2];   // the slot's bit in its half-block coverage word; 0 if unused
  uint32_t pix[2];   // ix | iy << 2 | sm << 4 | quad << 8 | pixel-in-quad << 10
  uint32_t zoff[2];  // offset of the slot in the staged depth, relative to the block
  float mx[2], my[2];  // sample position in the block
  float ax[2], ay[2];  // sample offset from the pixel centre (aa_z_offset)
};
__device__ inline LaneSlots lane_slots(TargetParams const& T, int lane, int zpitch) {
  LaneSlots ls;
  uint32_t const S = T.samples;
#pragma unroll
  for (int pass = 0; pass < 2; ++pass) {
    uint32_t slot = lane + 32 * pass;
    uint32_t i16 = slot / S, sm = slot % S;
    uint32_t ix = i16 & 3, iy = (i16 >> 2) & 3;
    uint32_t q = ((iy >> 1) << 1) | (ix >> 1), i = ((iy & 1) << 1) | (ix & 1);
    ls.bit[pass] = slot < 16 * S ? 1u << (4 * i + sm + 16 * (q & 1)) : 0u;
    ls.pix[pass] = ix | (iy << 2) | (sm << 4) | (q << 8) | (i << 10);
    ls.zoff[pass] = (iy * zpitch + ix) * S + sm;
    ls.mx[pass] = T.sp_x[sm & 3u] + static_cast<float>(ix);
    ls.my[pass] = T.sp_y[sm & 3u] + static_cast<float>(iy);
    ls.ax[pass] = T.sp_x[sm & 3u] - 0.5f;
    ls.ay[pass] = T.sp_y[sm & 3u] - 0.5f;
  }
  return ls;
}

// One (triangle, 4x4 block) pair processed by the whole warp: the block's
// level-2 classification (rasterizer.cpp:441-571), the per-sample coverage
// of draw_partial_tile (rasterizer.cpp:298-439) and early-Z
// (framebuffer.cpp:522-614) over the block's 16 pixels x samples, one sample
// slot per lane and pass; the quads' masks are assembled with warp
// reductions and the block's owner lane appends the surviving quads.
__device__ inline void pair_warp(PassParams const& P, TargetParams const& T, TriStage const* st, bool full16,
                                 int tile_x0, int tile_y0, int blk, int owner, OwnerList& L, uint32_t* ztile, int zx0,
                                 int zy0, int zpitch, LaneSlots const& ls, int lane) {
  StageView t{st};
  int const bx = blk & 15, by = blk >> 4;
  int const bx_abs = tile_x0 + bx * 4, by_abs = tile_y0 + by * 4;
  float const trr = T.target_w, trb = T.target_h;
  float4 e[3] = {t.edge(0), t.edge(1), t.edge(2)};
  bool region_full = full16;
  if (!full16) {
    LevelParams l1, l2;
    level_params(e, l1, l2);
    int r16x = tile_x0 + (bx >> 2) * 16, r16y = tile_y0 + (by >> 2) * 16;
    int c = child_class(e, l2, static_cast<float>(r16x), static_cast<float>(r16y), bx & 3, by & 3);
    if (c == 0) return;
    if (static_cast<float>(bx_abs) >= trr || static_cast<float>(by_abs) >= trb) return;
    region_full = c == 2;
  }
  uint32_t const W = T.width, H = T.height;
  float const lf = static_cast<float>(bx_abs), tf = static_cast<float>(by_abs);
  float ev[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) ev[k] = e[k].z - (lf * e[k].x + tf * e[k].y);
  // coverage: unclipped (uc) and clipped to the target (cv), 4 bits per pixel,
  // quads 0/1 in the low word, 2/3 in the high word
  uint32_t uc_lo = 0, uc_hi = 0, cv_lo = 0, cv_hi = 0;
#pragma unroll
  for (int pass = 0; pass < 2; ++pass) {
    uint32_t bit = ls.bit[pass];
    bool in = region_full;
    if (!in) {
      float mx = ls.mx[pass], my = ls.my[pass];
      bool rej = false;
#pragma unroll
      for (int k = 0; k < 3; ++k) rej = rej || ((mx * e[k].x + my * e[k].y) < ev[k]);
      in = !rej;
    }
    uint32_t pix = ls.pix[pass];
    bool hi = (pix >> 9) & 1u;
    // EXTENSION: pixels outside the target are not covered
    bool inside = bx_abs + (pix & 3u) < W && by_abs + ((pix >> 2) & 3u) < H;
    uint32_t ub = in ? bit : 0u, cb = in && inside ? bit : 0u;
    if (hi) {
      uc_hi |= ub;
      cv_hi |= cb;
    } else {
      uc_lo |= ub;
      cv_lo |= cb;
    }
  }
  uc_lo = __reduce_or_sync(0xFFFFFFFFu, uc_lo);
  uc_hi = __reduce_or_sync(0xFFFFFFFFu, uc_hi);
  cv_lo = __reduce_or_sync(0xFFFFFFFFu, cv_lo);
  cv_hi = __reduce_or_sync(0xFFFFFFFFu, cv_hi);
  if ((cv_lo | cv_hi) == 0) return;
  uint32_t const fm = (1u << T.samples) - 1u;
  uint32_t const qfull = fm | (fm << 4) | (fm << 8) | (fm << 12);
  // a full region's quads are drawn when their left / top pixel is inside the
  // target (draw_full_tile, rasterizer.cpp:738-742): no quad of this block is
  // dropped by that rule once its covered pixels are clipped to the target.
  uint32_t tested_lo = cv_lo, tested_hi = cv_hi;
  uint32_t const zc = st->zcfg;
  if (zc & 128u) {  // early-Z: depth test and write now, on the staged depth
    v4 v0 = t.v0(0);
    float dz = t.ddx(0).z, dyz = t.ddy(0).z;
    uint32_t t_lo = 0, t_hi = 0;
    uint32_t const func = (zc >> 8) & 15u;
    bool const rd = (zc >> 4) & 1u, wr = (zc >> 5) & 1u, d24 = (zc >> 6) & 1u;
    uint32_t* zblk = ztile + ((by_abs - zy0) * zpitch + (bx_abs - zx0)) * T.samples;
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
      uint32_t bit = ls.bit[pass], pix = ls.pix[pass];
      bool hi = (pix >> 9) & 1u;
      if (!((hi ? cv_hi : cv_lo) & bit)) continue;
      uint32_t q = (pix >> 8) & 3u, i = (pix >> 10) & 3u;
      uint32_t qx = bx_abs + ((q & 1) << 1), qy = by_abs + (q & 2);
      float dx = 0.5f + static_cast<float>(qx) - v0.x;
      float dy = 0.5f + static_cast<float>(qy) - v0.y;
      float z = quad_pos(t, dx, dy, static_cast<int>(i)).z;
      float nd = T.samples == 1 ? z : (ls.ax[pass] * dz + ls.ay[pass] * dyz) + z;
      uint32_t* zp = zblk + ls.zoff[pass];
      uint32_t w = *zp;
      bool pass_z = d24 ? cmpu(func, d24_quantize(nd), rd ? (w & 0xFFFFFFu) : 0u)
                        : cmpf(func, nd, rd ? __uint_as_float(w) : 0.0f);
      if (pass_z) {
        if (wr) *zp = d24 ? ((w & 0xFF000000u) | d24_quantize(nd)) : __float_as_uint(nd);
        if (hi) t_hi |= bit; else t_lo |= bit;
      }
    }
    tested_lo = __reduce_or_sync(0xFFFFFFFFu, t_lo);
    tested_hi = __reduce_or_sync(0xFFFFFFFFu, t_hi);
  }
  if (lane == owner) {
    uint32_t const rec = st->entry >> 1;
    uint32_t const na = st->shade_key << 25;
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
      uint32_t tq = ((q < 2 ? tested_lo : tested_hi) >> (16 * (q & 1))) & 0xFFFFu;
      if (!tq) continue;
      uint32_t cq = ((q < 2 ? cv_lo : cv_hi) >> (16 * (q & 1))) & 0xFFFFu;
      uint32_t uq = ((q < 2 ? uc_lo : uc_hi) >> (16 * (q & 1))) & 0xFFFFu;
      bool full = region_full ? cq == qfull : (uq == qfull && cq == uq);
      uint32_t qx = bx_abs + ((q & 1) << 1), qy = by_abs + (q & 2);
      owner_append(P, L, rec, (qx >> 1) | ((qy >> 1) << 12) | (full ? 1u << 24 : 0u) | na, tq | (cq << 16));
    }
  }
}

// Block owned by lane l < 4 n of warp w in an n x n-block item (n = 8 or 4):
// the blocks (x, y) with (x + y) mod 4 = w, so that the blocks along a row, a
// column or an anti-diagonal spread over all four warps.
__device__ inline void owned_block(int n, int w, int l, int& x, int& y) {
  if (n == 8) {
    y = l >> 1;
    x = ((w - y) & 3) + 4 * (l & 1);
  } else {
    y = l;
    x = (w - y) & 3;
  }
}

// Coverage of one pass.  Work items are squares of one tile: its four 32x32
// quadrants, or, for a tile with more than P.split_entries bin entries, its
// sixteen 16x16 regions, taken from a dynamic cursor over 16 item slots per
// tile.  A CTA stages the tile's triangles in batches, classifies them
// against the item's 16x16 regions and 4x4 blocks (rasterizer.cpp:441-571),
// and its four warps walk (triangle, block) pairs in primitive order with the
// item's depth held in shared memory for early-Z.
__global__ void __launch_bounds__(COVER_THREADS, 4) k_cover(PassParams P) {
  extern __shared__ __align__(16) uint8_t smem[];
  TriStage* stage = reinterpret_cast<TriStage*>(smem);
  // triangle sets of the staged batch (word-major): per 4x4 block of the item
  // (its 16x16 region partial, block inside the bounding box) and per 16x16
  // region of the item (region accepted)
  uint32_t* mask4 = reinterpret_cast<uint32_t*>(smem + STAGE_TRIS * sizeof(TriStage));
  uint32_t* mask16 = mask4 + 64 * MASK_WORDS;
  uint32_t* ztile = mask16 + 4 * MASK_WORDS;
  __shared__ uint32_t s_item;
  if ((P.counters->overflow & (OVF_BIN | OVF_REC)) || pass_gated(P)) return;
  int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t const nslots = P.ntiles * 16;
  OwnerList L{NO_CHUNK, NO_CHUNK, 0};
  for (;;) {
    if (tid == 0) s_item = atomicAdd(&P.counters->tile_cursor, 1u);
    __syncthreads();
    uint32_t const item = s_item;
    __syncthreads();
    if (item >= nslots) break;
    uint32_t const tile = item >> 4, sub = item & 15;
    uint32_t const begin = P.tile_begin[tile], end = P.tile_begin[tile + 1];
    bool const split = P.cover_item == 16 || end - begin > P.split_entries;
    if (!split && sub >= 4) continue;
    TargetParams const& T = P.targets[target_of_tile(P, tile)];
    uint32_t const ltile = tile - T.tile_base;
    int const n = split ? 4 : 8;   // blocks per side
    int const px = 4 * n;          // pixels per side
    int const rs = n >> 2;         // 16x16 regions per side
    int const bx0 = split ? (sub & 3) * 4 : (sub & 1) * 8, by0 = split ? (sub >> 2) * 4 : (sub >> 1) * 8;
    int const tile_x0 = static_cast<int>(ltile % T.tiles_x) * TILE, tile_y0 = static_cast<int>(ltile / T.tiles_x) * TILE;
    int const x0 = tile_x0 + bx0 * 4, y0 = tile_y0 + by0 * 4;
    int const r16x0 = bx0 >> 2, r16y0 = by0 >> 2;  // first 16x16 region of the item
    bool const owns = lane < (n == 8 ? 16 : 4);
    int ox = 0, oy = 0;
    owned_block(n, warp, lane & 15, ox, oy);
    int const blk = (by0 + oy) * 16 + bx0 + ox;           // owned block, tile numbering
    int const ib = oy * n + ox;                            // owned block, item numbering
    int const own16 = (oy >> 2) * rs + (ox >> 2);          // its 16x16 region, item numbering
    LaneSlots const ls = lane_slots(T, lane, px);
    float const tx0f = static_cast<float>(tile_x0), ty0f = static_cast<float>(tile_y0);
    float const trr = T.target_w, trb = T.target_h;
    uint32_t const S = T.samples;
    L.first = L.cur = NO_CHUNK;
    L.count = 0;
    bool const stage_z = T.any_early_z && begin < end;
    uint32_t const qw = min(static_cast<uint32_t>(px), T.width - min(T.width, static_cast<uint32_t>(x0)));
    uint32_t const qh = min(static_cast<uint32_t>(px), T.height - min(T.height, static_cast<uint32_t>(y0)));
    uint32_t const zrow = px * S;
    if (stage_z) {
      // the item's depth, and its pre-image for k_cover_rollback
      uint32_t* const zb = (P.zbackup && !T.zpre_known) ? P.zbackup + static_cast<size_t>(tile) * P.zbackup_tile_words +
                                           (static_cast<size_t>(by0) * 4 * TILE + bx0 * 4) * S
                                     : nullptr;
      for (uint32_t i = tid; i < qh * zrow; i += COVER_THREADS) {
        uint32_t y = i >> (__ffs(zrow) - 1), k = i & (zrow - 1);  // zrow: a power of two
        if (k >= qw * S) continue;
        uint32_t x = k >> (S >> 1), sm = k & (S - 1);
        uint32_t const v = *reinterpret_cast<uint32_t const*>(ds_addr(T, x0 + x, y0 + y, sm));
        ztile[i] = v;
        if (zb) zb[static_cast<size_t>(y) * TILE * S + k] = v;
      }
    }
    for (uint32_t bstart = begin; bstart < end; bstart += STAGE_TRIS) {
      uint32_t nb = min(static_cast<uint32_t>(STAGE_TRIS), end - bstart);
      __syncthreads();
      for (int i = tid; i < (64 + 4) * MASK_WORDS; i += COVER_THREADS) mask4[i] = 0;
      __syncthreads();
      // stage the batch and classify each triangle against the item's 16x16 regions
      for (uint32_t i = tid; i < nb; i += COVER_THREADS) {
        uint32_t e = P.bin_entries[bstart + i];
        float4 const* R = P.recs + (e >> 1);
        DrawParams const& D = P.draws[rec_draw(R)];
        int const nreg = 1 + static_cast<int>(D.nattr);
        TriStage ts;
        ts.e0 = R[0];
        ts.e1 = R[1];
        ts.e2 = R[2];
        ts.bbox = R[3];
        ts.p0 = R[5];
        ts.dpx = R[5 + nreg];
        ts.dpy = R[5 + 2 * nreg];
        ts.entry = e;
        ts.zcfg = D.zcfg;
        ts.shade_key = D.shade_key;
        ts.pad = 0;
        stage[i] = ts;
        uint32_t bit = 1u << (i & 31), word = i >> 5;
        if (e & 1u) {  // accepted for the whole tile by the binner
          for (int r = 0; r < rs * rs; ++r) atomicOr(&mask16[word * 4 + r], bit);
          continue;
        }
        float x_min = ts.bbox.x - tx0f, x_max = ts.bbox.y - tx0f, y_min = ts.bbox.z - ty0f, y_max = ts.bbox.w - ty0f;
        float4 ed[3] = {ts.e0, ts.e1, ts.e2};
        LevelParams l1, l2;
        level_params(ed, l1, l2);
        for (int iy = r16y0; iy < r16y0 + rs; ++iy) {
          int m16y = iy * 16;
          if (y_min >= static_cast<float>(m16y + 16) || y_max < static_cast<float>(m16y)) continue;
          for (int ix = r16x0; ix < r16x0 + rs; ++ix) {
            int m16x = ix * 16;
            if (x_min >= static_cast<float>(m16x + 16) || x_max < static_cast<float>(m16x)) continue;
            int c = child_class(ed, l1, tx0f, ty0f, ix, iy);
            if (c == 0) continue;
            // a region whose origin is right of / below the target is skipped
            if (static_cast<float>(tile_x0 + m16x) >= trr || static_cast<float>(tile_y0 + m16y) >= trb) continue;
            if (c == 2) {
              atomicOr(&mask16[word * 4 + (iy - r16y0) * rs + (ix - r16x0)], bit);
              continue;
            }
            // partial: the 4x4 children that pass the level-2 bounding-box test
            for (int jy = 0; jy < 4; ++jy) {
              int m4y = m16y + jy * 4;
              if (y_min >= static_cast<float>(m4y + 4) || y_max < static_cast<float>(m4y)) continue;
              for (int jx = 0; jx < 4; ++jx) {
                int m4x = m16x + jx * 4;
                if (x_min >= static_cast<float>(m4x + 4) || x_max < static_cast<float>(m4x)) continue;
                atomicOr(&mask4[word * 64 + (iy * 4 + jy - by0) * n + (ix * 4 + jx - bx0)], bit);
              }
            }
          }
        }
      }
      __syncthreads();
      // Each warp walks the batch's triangles in primitive order and, for
      // each, the owned blocks the triangle reaches, processing every
      // (triangle, block) pair with the whole warp; per block this is the
      // reference's primitive order.
      for (int w = 0; w < MASK_WORDS; ++w) {
        uint32_t m16 = owns ? mask16[w * 4 + own16] : 0u;
        uint32_t mine = owns ? (mask4[w * 64 + ib] | m16) : 0u;
        uint32_t tris = __reduce_or_sync(0xFFFFFFFFu, mine);
        while (tris) {
          int b = __ffs(tris) - 1;
          tris &= tris - 1;
          uint32_t blocks = __ballot_sync(0xFFFFFFFFu, (mine >> b) & 1u);
          uint32_t fulls = __ballot_sync(0xFFFFFFFFu, (m16 >> b) & 1u);
          while (blocks) {
            int l = __ffs(blocks) - 1;
            blocks &= blocks - 1;
            int lx, ly;
            owned_block(n, warp, l, lx, ly);
            int oblk = (by0 + ly) * 16 + bx0 + lx;
            pair_warp(P, T, stage + (w << 5) + b, (fulls >> l) & 1u, tile_x0, tile_y0, oblk, l, L, ztile, x0, y0,
                      px, ls, lane);
          }
        }
      }
    }
    if (stage_z) {
      __syncthreads();
      for (uint32_t i = tid; i < qh * zrow; i += COVER_THREADS) {
        uint32_t y = i >> (__ffs(zrow) - 1), k = i & (zrow - 1);  // zrow: a power of two
        if (k >= qw * S) continue;
        uint32_t x = k >> (S >> 1), sm = k & (S - 1);
        *reinterpret_cast<uint32_t*>(ds_addr(T, x0 + x, y0 + y, sm)) = ztile[i];
      }
    }
    // close the owned block's list for the item
    if (owns) {
      if (L.cur != NO_CHUNK) {
        P.chunk_next[L.cur] = NO_CHUNK;
        P.chunk_count[L.cur] = L.count;
      }
      // the block's whole list goes to the owner of its top-left quad; the
      // block's other quads have none
      uint32_t* const of = P.owner_first + static_cast<size_t>(tile) * QUAD_OWNERS + (blk >> 4) * 64 + (blk & 15) * 2;
      of[0] = L.first;
      of[1] = NO_CHUNK;
      of[32] = NO_CHUNK;
      of[33] = NO_CHUNK;
    }
  }
}

#endif  // SG_RASTER_COVER_MERGE

// cpp_pixel_shader programs for one pixel `q` of a quad shaded by four lanes
// (lanes 4k..4k+3 of the warp); ddx / ddy are the quad differences and
// tex2d's LOD uses them (cpp_pixel_shader.cpp:13-31).  `keep` is the
// program's return value: false discards the pixel.
// Attribute 0 at the quad's pixels 0, 1 (x + 1) and 2 (y + 1), from which
// the programs take ddx / ddy: read from the quad's lanes by shuffles.
struct QuadNb {
  int base;
  unsigned mask;
  float a0w;
  float u0, v0, u1, v1, u2, v2;
  __device__ explicit QuadNb(v4 a0) {
    base = (threadIdx.x & 31) & ~3;
    mask = 0xFu << base;
    a0w = a0.w;
    u0 = __shfl_sync(mask, a0.x, base);
    v0 = __shfl_sync(mask, a0.y, base);
    u1 = __shfl_sync(mask, a0.x, base + 1);
    v1 = __shfl_sync(mask, a0.y, base + 1);
    u2 = __shfl_sync(mask, a0.x, base + 2);
    v2 = __shfl_sync(mask, a0.y, base + 2);
  }
  __device__ float w(int i) const { return __shfl_sync(mask, a0w, base + i); }  // every lane of the quad calls it
};
// The same for one pixel of a line: the pixel and its neighbours one ddx /
// one ddy along the line, given.
struct LineNb {
  float u0, v0, u1, v1, u2, v2;
  float ws[3];
  __device__ float w(int i) const { return ws[i]; }
};

// INL: the sampler inlined (sample_impl_sel)
template <int NA, class NB, bool INL = false>
__device__ inline v4 run_ps_nb(DrawParams const& D, v4 const* attr, NB const& nb, bool& keep) {
  v4 a0 = NA > 0 ? attr[0] : mk4(0, 0, 0, 0);
  v4 a1 = NA > 1 ? attr[1 < NA ? 1 : 0] : mk4(0, 0, 0, 0);
  float const u0 = nb.u0, v0 = nb.v0, u1 = nb.u1, v1 = nb.v1, u2 = nb.u2, v2 = nb.v2;
  keep = true;
  switch (D.ps_prog) {
  case SG_PS_COLOR:
  case SG_PS_COLOR_MRT: return a0;  // (its other colours: k_shade)
  case SG_PS_CONSTANT: return mk4(D.ps_k[0], D.ps_k[1], D.ps_k[2], D.ps_k[3]);
  case SG_PS_TEX_MODULATE: {
    float lod = calc_lod_2d(D.ps_samp, u1 - u0, v1 - v0, u2 - u0, v2 - v0);
    return mulv(sample_impl_sel<INL>(D.ps_samp, a0.x, a0.y, lod, nullptr), a1);
  }
  case SG_PS_TEX_GRAD_MODULATE:
  case SG_PS_TEX_GRAD_LEARNED:  // the lookups the learned filter does not take
    return mulv(sample_2d_grad<INL>(D.ps_samp, a0.x, a0.y, u1 - u0, v1 - v0, u2 - u0, v2 - v0, 0.0f), a1);
  case SG_PS_TEX_LOD_MODULATE:  // tex2dlod(s, 0) = s.sample(x, y, w) (cpp_pixel_shader.cpp:33-40)
    return mulv(sample_impl_sel<INL>(D.ps_samp, a0.x, a0.y, a0.w, nullptr), a1);
  case SG_PS_TEX_PROJ_MODULATE: {  // tex2dproj(s, 0) (cpp_pixel_shader.cpp:42-60)
    float const w0 = nb.w(0), w1 = nb.w(1), w2 = nb.w(2);
    // this pixel's attribute, and it stepped by ddx and by ddy
    float const nxx = a0.x + (u1 - u0), nxy = a0.y + (v1 - v0), nxw = a0.w + (w1 - w0);
    float const nyx = a0.x + (u2 - u0), nyy = a0.y + (v2 - v0), nyw = a0.w + (w2 - w0);
    float const px = (a0.x / a0.w + 1.0f) * 0.5f, py = (a0.y / a0.w + 1.0f) * 0.5f;
    float const qxx = (nxx / nxw + 1.0f) * 0.5f, qxy = (nxy / nxw + 1.0f) * 0.5f;
    float const qyx = (nyx / nyw + 1.0f) * 0.5f, qyy = (nyy / nyw + 1.0f) * 0.5f;
    return mulv(sample_2d_grad<INL>(D.ps_samp, px, py, qxx - px, qxy - py, qyx - px, qyy - py, 0.0f), a1);
  }
  case SG_PS_TEXCUBE_MODULATE:  // sampler::sample_cube(x, y, z, w) (sampler.cpp:771-829)
    return mulv(sample_cube(D.ps_samp, a0.x, a0.y, a0.z, a0.w), a1);
  case SG_PS_TEX_ALPHA_TEST: {  // tex2d * attr[1], discarded below constants[0] alpha
    float lod = calc_lod_2d(D.ps_samp, u1 - u0, v1 - v0, u2 - u0, v2 - v0);
    v4 const c = mulv(sample_impl_sel<INL>(D.ps_samp, a0.x, a0.y, lod, nullptr), a1);
    keep = !(c.w < D.ps_k[0]);
    return c;
  }
  default: return mk4(0, 0, 0, 0);
  }
}
template <int NA, bool INL = false>
__device__ inline v4 run_ps(DrawParams const& D, v4 const* attr, int, bool& keep) {
  QuadNb const nb(NA > 0 ? attr[0] : mk4(0, 0, 0, 0));
  return run_ps_nb<NA, QuadNb, INL>(D, attr, nb, keep);
}


// Whether the learned filter takes an SG_PS_TEX_GRAD_LEARNED lookup: a
// minified lookup of an anisotropic sampler whose probe count is above
// constants[2] and at most constants[1].
__device__ inline bool af_takes(DrawParams const& D, float dxu, float dxv, float dyu, float dyv, af_info& af) {
  dev_sampler const& s = D.ps_samp;
  if (s.mip_filter != SG_FILTER_ANISOTROPIC || s.max_anisotropy <= 1) return false;
  calc_af(s, dxu, dxv, dyu, dyv, 0.0f, af);
  return af.lod >= 0.0f && af.probe_count > D.ps_k[2] && af.probe_count <= D.ps_k[1];
}

// Attribute interpolation (step_2d_unproj_attr_n_quad / step_2d_unproj_attr_n
// with the centroid adjustment, shader.cpp:208-367, rasterizer.cpp:1363-1398)
// and the pixel shader, for every fragment of the pass whose draw has NA
// varyings.  The LEARNED instances take the SG_PS_TEX_GRAD_LEARNED draws
// (shade class 8 + NA) and queue the lookups the learned filter applies to;
// they wait mostly on texture taps and queue atomics, so they run 4 CTAs per
// SM (64 registers) where the plain instances run 3.
template <int NA, bool LEARNED, int MINB = (LEARNED ? 4 : 3)>
__global__ void __launch_bounds__(256, MINB) k_shade(PassParams P) {
  pdl_wait();
  if ((P.counters->overflow & OVF_FATAL) || pass_gated(P)) return;
  uint32_t const nfrag = min(P.counters->chunk_total, P.chunk_capacity) * FRAG_CHUNK;
  int const q = threadIdx.x & 3;
  uint32_t const groups = gridDim.x * (blockDim.x >> 2);
  uint32_t const start = blockIdx.x * (blockDim.x >> 2) + (threadIdx.x >> 2);
  // this instance's shade classes: NA varyings, plus 8 for learned-filter
  // draws; without a lookup queue the plain instances shade those draws too.
  // With the class lists, only their fragments are walked; else every slot.
  uint32_t const cls_a = LEARNED ? NA + 8u : NA;
  bool const with_b = !LEARNED && !P.af_capacity;
  uint32_t base_a = 0, n_a = 0, base_b = 0, n_b = 0;
  if (P.frag_list) {
    for (uint32_t key = 0; key < 128; ++key) {  // class c: keys [8c, 8c + 8)
      uint32_t const k = P.class_counts[key], c = key >> 3;
      if (c < cls_a) base_a += k;
      if (c == cls_a) n_a += k;
      if (c < NA + 8u) base_b += k;
      if (with_b && c == NA + 8u) n_b += k;
    }
  }
  uint32_t const total = P.frag_list ? n_a + n_b : nfrag;
  uint32_t const rounds = (total + groups - 1) / groups;
  // learned instances: each thread's network record (feature row and tap
  // mean) waits here, unit-major, until the warp has its queue slots
  __shared__ uint4 s_net[LEARNED ? 5 * 256 : 1];
  for (uint32_t it = 0; it < rounds; ++it) {
    uint32_t const idx = start + it * groups;
    uint32_t f;
    bool live;
    if (P.frag_list) {
      live = idx < total;
      f = live ? P.frag_list[idx < n_a ? base_a + idx : base_b + (idx - n_a)] : 0u;
    } else {
      f = idx;
      live = f < nfrag && (f % FRAG_CHUNK) < P.chunk_count[f / FRAG_CHUNK];
    }
    uint32_t pos = live ? P.frag_pos[f] : 0u;
    uint32_t const cls = frag_class(pos);
    live = live && (cls == cls_a || (with_b && cls == NA + 8u));
    uint32_t draw = 0xFFFFFFFFu;
    // learned instances: the pixel's lookup, for the network's queue (af_net)
    // or for the plain sampler's (af_plain)
    bool af_net = false, af_plain = false;
    float4 af_r0, af_r1, af_r2;
    if (live) {
      uint32_t rec = P.frag_rec[f], masks = P.frag_mask[f];
      TriView t{P.recs + rec, 1 + NA};
      draw = rec_draw(t.R);
      DrawParams const& D = P.draws[draw];
      TargetParams const& T = P.targets[D.target];
      v4 attr[NA > 0 ? NA : 1];
#pragma unroll
      for (int i = 0; i < (NA > 0 ? NA : 1); ++i) attr[i] = mk4(0, 0, 0, 0);
      uint32_t qx = (pos & 0xFFFu) << 1, qy = ((pos >> 12) & 0xFFFu) << 1;
      bool full = (pos >> 24) & 1u;
      v4 v0p = t.v0(0);
      float dx = 0.5f + static_cast<float>(qx) - v0p.x;
      float dy = 0.5f + static_cast<float>(qy) - v0p.y;
      float w = quad_pos(t, dx, dy, q).w;
      float invw = 1.0f / w;
      bool centroid = !full && D.has_centroid;
      float pdx = dx, pdy = dy;
      if (centroid) {
        pdx = dx + static_cast<float>(q & 1);
        pdy = dy + static_cast<float>(q >> 1);
        uint64_t m = expand_mask(masks >> 16);  // coverage before early-Z (rasterizer.cpp:1373)
        uint32_t pm = static_cast<uint32_t>(m >> (16 * q)) & 0xFFFFu;
        uint32_t fm = (1u << T.samples) - 1u;
        if (pm != fm && pm != 0) {
          float cx = 0.0f, cy = 0.0f;
          int n = 0;
          for (uint32_t s = 0; s < T.samples; ++s)
            if (pm & (1u << s)) {
              cx += T.sp_x[s];
              cy += T.sp_y[s];
              ++n;
            }
          float inv = 1.0f / static_cast<float>(n);
          cx *= inv;
          cy *= inv;
          pdx += cx - 0.5f;
          pdy += cy - 0.5f;
        }
      }
#pragma unroll
      for (int i = 0; i < NA; ++i) {
        v4 in = t.v0(1 + i), d0 = t.ddx(1 + i), d1 = t.ddy(1 + i);
        v4 a;
        if (D.mods[i] & SG_AM_NOINTERPOLATION) {
          a = in;
        } else if (centroid) {
          a = mk4(in.x + (d0.x * pdx + d1.x * pdy), in.y + (d0.y * pdx + d1.y * pdy), in.z + (d0.z * pdx + d1.z * pdy),
                  in.w + (d0.w * pdx + d1.w * pdy));
        } else {
          v4 a00 = mk4(in.x + (d0.x * dx + d1.x * dy), in.y + (d0.y * dx + d1.y * dy), in.z + (d0.z * dx + d1.z * dy),
                       in.w + (d0.w * dx + d1.w * dy));
          a = q == 0 ? a00 : q == 1 ? a00 + d0 : q == 2 ? a00 + d1 : (a00 + d0) + d1;
        }
        attr[i] = (D.mods[i] & SG_AM_NOPERSPECTIVE) ? a : a * invw;
      }
      if constexpr (LEARNED) {
        // the lookup, with the quad's derivatives as run_ps takes them (the
        // same for its four lanes, so a quad goes to one queue whole)
        int const base = (threadIdx.x & 31) & ~3;
        unsigned const qm = 0xFu << base;
        v4 const a0 = attr[0];
        float const u0 = __shfl_sync(qm, a0.x, base), v0 = __shfl_sync(qm, a0.y, base);
        float const u1 = __shfl_sync(qm, a0.x, base + 1), v1 = __shfl_sync(qm, a0.y, base + 1);
        float const u2 = __shfl_sync(qm, a0.x, base + 2), v2 = __shfl_sync(qm, a0.y, base + 2);
        af_info af;
        af_net = af_takes(D, u1 - u0, v1 - v0, u2 - u0, v2 - v0, af);
        af_plain = !af_net;
        if (af_net) {  // the network's features: taps by the texture units, BF16 for the tensor cores
          float fe[AF_F];
          af_features_from(D.ps_samp, a0.x, a0.y, u1 - u0, v1 - v0, u2 - u0, v2 - v0, af, fe);
          uint32_t w[16];
#pragma unroll
          for (int i = 0; i < 12; ++i)
            w[i] = static_cast<uint32_t>(__bfloat16_as_ushort(__float2bfloat16_rn(fe[2 * i]))) |
                   (static_cast<uint32_t>(__bfloat16_as_ushort(__float2bfloat16_rn(fe[2 * i + 1]))) << 16);
#pragma unroll
          for (int i = 12; i < 16; ++i) w[i] = 0u;
          if constexpr (LEARNED) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
              s_net[i * 256 + threadIdx.x] = make_uint4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
            s_net[4 * 256 + threadIdx.x] = make_uint4(__float_as_uint(af_skip(fe, 0)), __float_as_uint(af_skip(fe, 1)),
                                                      __float_as_uint(af_skip(fe, 2)), __float_as_uint(af_skip(fe, 3)));
          }
        }
        af_r0 = make_float4(a0.x, a0.y, u1 - u0, v1 - v0);
        af_r1 = make_float4(u2 - u0, v2 - v0, __uint_as_float(f * 4 + q), __uint_as_float(draw));
        v4 const m = NA > 1 ? attr[NA > 1 ? 1 : 0] : mk4(0, 0, 0, 0);
        af_r2 = make_float4(m.x, m.y, m.z, m.w);
        if (q == 0) P.frag_ps[f] = 0xF;  // the learned filter's lookups never discard
        if (P.frag_color_more)  // colours the program does not write are zero
          for (uint32_t i = 0; i < P.more_colors; ++i)
            P.frag_color_more[(static_cast<size_t>(f) * 4 + q) * P.more_colors + i] = make_float4(0, 0, 0, 0);
      } else {
        bool keep = true;
        // all four lanes of a quad take the same path; the 80-register
        // instances inline the sampler, the 64-register ones call it
        v4 out = run_ps<NA, (MINB <= 3)>(D, attr, q, keep);
        P.frag_color[static_cast<size_t>(f) * 4 + q] = make_float4(out.x, out.y, out.z, out.w);
        if (P.frag_color_more)  // colours 1..: attributes 1.. of SG_PS_COLOR_MRT, else zero
          for (uint32_t i = 0; i < P.more_colors; ++i) {
            v4 c = mk4(0, 0, 0, 0);
#pragma unroll
            for (int k = 1; k < NA; ++k)
              if (D.ps_prog == SG_PS_COLOR_MRT && static_cast<uint32_t>(k) == i + 1) c = attr[k];
            P.frag_color_more[(static_cast<size_t>(f) * 4 + q) * P.more_colors + i] = make_float4(c.x, c.y, c.z, c.w);
          }
        // the quad's pass mask as cpp_pixel_shader::execute builds it
        // (cpp_pixel_shader.cpp:62-74): from int shifts of 0xFFFF by 16 i, so
        // pixel 0 is kept when pixel 0 or 2 passes and pixels 1-3 when pixel
        // 1 or 3 passes (a negative int sign-extends, a 32-bit shift count wraps)
        int const qb = (threadIdx.x & 31) & ~3;
        uint32_t const passed = (__ballot_sync(0xFu << qb, keep) >> qb) & 0xFu;
        uint32_t const kept = ((passed & 5u) ? 1u : 0u) | ((passed & 10u) ? 14u : 0u);
        if (q == 0) P.frag_ps[f] = static_cast<uint8_t>(kept);
      }
    }
    if constexpr (LEARNED) {
      // queue the lookups, one atomic per warp and queue; lookups past the
      // network queue's end go to the plain queue (sized for the pass's
      // fragments; past its end the pass reports OVF_AF_QUEUE)
      int const lane = threadIdx.x & 31;
      unsigned const want_net = __ballot_sync(0xFFFFFFFFu, af_net);
      if (want_net) {
        int const leader = __ffs(want_net) - 1;
        uint32_t first = 0;
        if (lane == leader) first = atomicAdd(&P.counters->af_lookups, static_cast<unsigned>(__popc(want_net)));
        uint32_t const k = __shfl_sync(0xFFFFFFFFu, first, leader) + __popc(want_net & ((1u << lane) - 1u));
        if (af_net) {
          if (k < P.af_net_capacity) {
            uint4* x = reinterpret_cast<uint4*>(P.af_net + static_cast<size_t>(k) * AF_NET_UNITS);
#pragma unroll
            for (int i = 0; i < 5; ++i) x[i] = s_net[i * 256 + threadIdx.x];
            float4* r = P.af_net + static_cast<size_t>(k) * AF_NET_UNITS + 4;
            r[1] = af_r0;
            r[2] = af_r1;
            r[3] = af_r2;
          } else {
            af_plain = true;
          }
        }
      }
      unsigned const want_plain = __ballot_sync(0xFFFFFFFFu, af_plain);
      if (want_plain) {
        int const leader = __ffs(want_plain) - 1;
        uint32_t first = 0;
        if (lane == leader) first = atomicAdd(&P.counters->af_plain, static_cast<unsigned>(__popc(want_plain)));
        uint32_t const k = __shfl_sync(0xFFFFFFFFu, first, leader) + __popc(want_plain & ((1u << lane) - 1u));
        if (af_plain) {
          if (k < P.af_capacity) {
            float4* r = P.af_plain + static_cast<size_t>(k) * AF_PLAIN_UNITS;
            r[0] = af_r0;
            r[1] = af_r1;
            r[2] = af_r2;
          } else {
            atomicOr(&P.counters->overflow, OVF_AF_QUEUE);
          }
        }
      }
    }
    // ps_invocations: 4 per quad, counted per draw (one lane per quad)
    uint32_t key = q == 0 ? draw : 0xFFFFFFFFu;
    uint32_t grp = __match_any_sync(0xFFFFFFFFu, key);
    if (key != 0xFFFFFFFFu && (threadIdx.x & 31) == static_cast<uint32_t>(__ffs(grp) - 1))
      atomicAdd(&P.draw_stats[key].ps_invocations, 4ull * static_cast<unsigned>(__popc(grp)));
  }
}

// Output merging: owners replay their fragments in primitive order
// (framebuffer::render_sample_quad, framebuffer.cpp:481-520).
// Work is handed out per warp -- 32 owners of a tile at a time, from a
// device-wide cursor -- so tiles of very different cost spread over the SMs.
// UBS: a user blend shader the pass's user-blend draws run (void: none).
template <class UBS>
__device__ __forceinline__ void merge_pass(PassParams const& P) {
  pdl_wait();
  if (pass_gated(P)) return;
  uint32_t const ovf = P.counters->overflow;  // final: geometry, binning, coverage and shading are done
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (ovf) atomicOr(P.sticky, ovf);
    if (P.count_pass && !(ovf & OVF_FATAL)) atomicAdd(P.sticky + 1, 1u);
  }
  if (ovf & OVF_FATAL) return;
  int const lane = threadIdx.x & 31;
  uint32_t const groups = QUAD_OWNERS / 32;  // owner groups per tile
  uint32_t cur_draw = 0xFFFFFFFFu;
  unsigned long long backend = 0;
  for (;;) {
    uint32_t unit = 0;
    if (lane == 0) unit = atomicAdd(&P.counters->merge_cursor, 1u);
    unit = __shfl_sync(0xFFFFFFFFu, unit, 0);
    if (unit / groups >= P.ntiles) break;
    uint32_t const tile = P.tile_order ? P.tile_order[unit / groups] : unit / groups;
    uint32_t const owner = (unit % groups) * 32 + lane;
    uint32_t c = P.tile_begin[tile] == P.tile_begin[tile + 1]
                     ? NO_CHUNK
                     : P.owner_first[static_cast<size_t>(tile) * QUAD_OWNERS + owner];
    // the next fragment's header and record flags are read a fragment ahead
    // (they are read-only here), overlapping their latency with the blend
    uint32_t n = c != NO_CHUNK ? __ldg(&P.chunk_count[c]) : 0u, k = 0;
    uint32_t h_rec = 0, h_pos = 0, h_mask = 0, h_ps = 0, h_draw = 0;
    if (n) {
      uint32_t const f0 = c * FRAG_CHUNK;
      h_rec = __ldg(&P.frag_rec[f0]);
      h_pos = __ldg(&P.frag_pos[f0]);
      h_mask = __ldg(&P.frag_mask[f0]);
      h_ps = __ldg(&P.frag_ps[f0]);
      h_draw = __float_as_uint(__ldg(&P.recs[h_rec + 4].z));
    }
    while (c != NO_CHUNK) {
      {
        uint32_t const f = c * FRAG_CHUNK + k;
        uint32_t const rec = h_rec, pos = h_pos, masks = h_mask, ps = h_ps, rdraw = h_draw;
        // advance to the next fragment and start its loads
        if (++k == n) {
          c = __ldg(&P.chunk_next[c]);
          k = 0;
          n = c != NO_CHUNK ? __ldg(&P.chunk_count[c]) : 0u;
        }
        if (c != NO_CHUNK && k < n) {
          uint32_t const fn = c * FRAG_CHUNK + k;
          h_rec = __ldg(&P.frag_rec[fn]);
          h_pos = __ldg(&P.frag_pos[fn]);
          h_mask = __ldg(&P.frag_mask[fn]);
          h_ps = __ldg(&P.frag_ps[fn]);
          h_draw = __float_as_uint(__ldg(&P.recs[h_rec + 4].z));
        }
        uint64_t m = expand_mask(masks & 0xFFFFu);
        uint64_t psm = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (ps & (1u << i)) psm |= 0xFFFFull << (16 * i);
        m &= psm;
        bool full = (pos >> 24) & 1u;
        if (full && m == 0) continue;
        float4 const* R = P.recs + rec;
        uint32_t const draw = rdraw;
        if (draw != cur_draw) {
          if (backend) atomicAdd(&P.draw_stats[cur_draw].backend_input_pixels, backend);
          backend = 0;
          cur_draw = draw;
        }
        backend += 4;
        DrawParams const& D = P.draws[draw];
        TargetParams const& T = P.targets[D.target];
        TriView t{R, 1 + static_cast<int>(D.nattr)};
        uint32_t qx = (pos & 0xFFFu) << 1, qy = ((pos >> 12) & 0xFFFu) << 1;
        bool front = t.front();
        float depth[4] = {0, 0, 0, 0};
        float aa[4] = {0, 0, 0, 0};
        if (!D.early_z && T.ds) {
          v4 v0p = t.v0(0);
          float dx = 0.5f + static_cast<float>(qx) - v0p.x;
          float dy = 0.5f + static_cast<float>(qy) - v0p.y;
#pragma unroll
          for (int i = 0; i < 4; ++i) depth[i] = quad_pos(t, dx, dy, i).z;
          if (T.samples > 1) {
            float dz = t.ddx(0).z, dyz = t.ddy(0).z;
            for (uint32_t s = 0; s < T.samples; ++s) aa[s] = (T.sp_x[s] - 0.5f) * dz + (T.sp_y[s] - 0.5f) * dyz;
          }
        }
        if ((D.early_z || !T.ds) && T.color && T.color_esz == 4 && T.samples == 4 &&
            (T.nmore == 0 || D.bs_prog != SG_BS_REPLACE_ALL) && D.bs_prog < SG_USER_PROGRAM_BASE) {
          // colour only, four 4-byte samples per pixel: each covered pixel's
          // samples are read, blended and written as one 16-byte word
          uint4 w[4];
          float4 cc[4];
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if ((m >> (16 * i)) & 0xFu) {
              uint32_t x = qx + (i & 1), y = qy + (i >> 1);
              w[i] = *reinterpret_cast<uint4 const*>(color_addr(T, x, y, 0));
              cc[i] = P.frag_color[static_cast<size_t>(f) * 4 + i];
            }
          // the blend with the format and program as constants for the
          // common state (RGBA8, source-alpha lerp), else as data
          auto blend_quad = [&](uint32_t fmt, uint32_t bs) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              uint32_t const pm = static_cast<uint32_t>(m >> (16 * i)) & 0xFu;
              if (!pm) continue;
              v4 const src = mk4(cc[i].x, cc[i].y, cc[i].z, cc[i].w);
              if (pm & 1u) w[i].x = blend_word(fmt, bs, w[i].x, src);
              if (pm & 2u) w[i].y = blend_word(fmt, bs, w[i].y, src);
              if (pm & 4u) w[i].z = blend_word(fmt, bs, w[i].z, src);
              if (pm & 8u) w[i].w = blend_word(fmt, bs, w[i].w, src);
              uint32_t x = qx + (i & 1), y = qy + (i >> 1);
              *reinterpret_cast<uint4*>(color_addr(T, x, y, 0)) = w[i];
            }
          };
          if (T.color_fmt == SG_FMT_RGBA8 && D.bs_prog == SG_BS_LERP_SRC_ALPHA)
            blend_quad(SG_FMT_RGBA8, SG_BS_LERP_SRC_ALPHA);
          else
            blend_quad(T.color_fmt, D.bs_prog);
          continue;
        }
        for (int i = 0; i < 4; ++i) {
          uint32_t pm = static_cast<uint32_t>(m >> (16 * i)) & 0xFFFFu;
          if (!pm) continue;
          float4 cc = P.frag_color[static_cast<size_t>(f) * 4 + i];
          v4 src = mk4(cc.x, cc.y, cc.z, cc.w);
          float4 const* more =
              P.frag_color_more ? P.frag_color_more + (static_cast<size_t>(f) * 4 + i) * P.more_colors : nullptr;
          uint32_t x = qx + (i & 1), y = qy + (i >> 1);
          if (T.samples == 1) {
            render_sample<UBS>(T, D, x, y, 0, src, depth[i], front, more);
          } else {
            for (uint32_t s = 0; s < T.samples; ++s)
              if (pm & (1u << s)) render_sample<UBS>(T, D, x, y, s, src, depth[i] + aa[s], front, more);
          }
        }
      }
    }
  }
  if (backend) atomicAdd(&P.draw_stats[cur_draw].backend_input_pixels, backend);
}

#ifdef SG_RASTER_COVER_MERGE
// MINB: CTAs per SM the registers are cut for (3: 80 registers, no spills;
// 4: 64, with spills) -- a tuning choice
template <int MINB>
__global__ void __launch_bounds__(RASTER_THREADS, MINB) k_merge(PassParams P) { merge_pass<void>(P); }

#endif  // SG_RASTER_COVER_MERGE

// ---------------------------------------------------------------------------
// `resident`: CTAs per SM the plain instances' registers are cut for (3 or 4)
template <int NA>
void launch_shade_t(PassParams const& P, uint32_t grid, uint32_t resident, cudaStream_t s) {
  if (resident >= 4)
    launch_pdl(k_shade<NA, false, 4>, grid, 256, 0, s, P);
  else
    launch_pdl(k_shade<NA, false, 3>, grid, 256, 0, s, P);
}
template <int NA>
void launch_shade_learned_t(PassParams const& P, uint32_t grid, cudaStream_t s) {
  launch_pdl(k_shade<NA, true>, grid, 256, 0, s, P);
}

}  // namespace sg
