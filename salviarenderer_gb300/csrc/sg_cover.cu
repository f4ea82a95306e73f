// sg_cover.cu -- coverage and early-Z of a pass.
//
// Work items are the 32x32 quadrants of every tile of every target, taken
// from a dynamic cursor (costliest tiles first); a CTA of 256 threads
// handles one item at a time, four threads per 4x4 block, one per 2x2 quad.
// For each batch of the tile's triangles (its bin list, in API order) the
// CTA
//   1. stages the batch -- the next CV_STAGE of the tile's triangles whose
//      bounding box reaches the quadrant, compacted in order from the bin
//      list -- and classifies every staged triangle against the
//      quadrant's 16x16 regions and 4x4 blocks with the reference's level-1
//      and level-2 trivial reject / accept tests (rasterizer.cpp:441-571),
//      into per-block sets of the triangles reaching the block and of those
//      covering it fully;
//   2. drops, per block, the triangles a hierarchical depth test proves
//      hidden (below);
//   3. in rounds of up to CV_K triangles per block: computes the per-sample
//      coverage of every remaining (triangle, block) pair -- the edge test of
//      draw_partial_tile, rasterizer.cpp:298-439 -- spread evenly over all
//      threads (coverage does not depend on order), then lets each of the
//      block's four threads walk its pairs in primitive order on its quad:
//      early-Z (framebuffer.cpp:522-614) on the quad's samples against the
//      quadrant's depth staged in shared memory, and the surviving quad
//      appended to that quad's own fragment list.  Quads are disjoint, so
//      the four walks need no synchronisation.  The common depth functions
//      (LESS, LESS_EQUAL on float or D24 storage) run as compiled compares,
//      chosen once per pair; the others go through the general compare.
//
// Hierarchical depth test: the block's four threads keep the largest and
// smallest depth stored in the block, recomputed at the start of each batch
// after writes.  A triangle's depth over the block is bounded from its depth
// plane, widened by a margin that covers the rounding of the reference's
// per-sample depth expression; when the bound proves every sample of the
// block fails the depth test, the pair is dropped (the four threads test a
// quarter of the block's triangles each).  Such samples neither pass nor
// write, so results are those of testing every sample.  The depth range only
// narrows toward passing values as samples are written, so a drop decided at
// the start of a batch stays right for the whole batch.
#include "sg_raster.cuh"

namespace sg {

constexpr int CV_THREADS = 256;              // 64 blocks x 4 quads
constexpr int CV_STAGE = 128;                // triangles per staged batch
constexpr int CV_WORDS = CV_STAGE / 32;
constexpr int CV_PX = 32;                    // quadrant edge
constexpr int CV_K = 16;                     // pairs per block per round

struct TriCv {  // what coverage and early-Z read of a triangle
  float4 e0, e1, e2, bbox;
  float p0x, p0y, p0z, dzx;
  float dzy;
  uint32_t entry, zcfg, shade_key;  // shade class * 8 + pixel-shader program
};

// Shared memory of one CTA.
struct CvShared {
  TriCv stage[CV_STAGE];
  // per word of the batch, one bit per staged triangle: reaching each block,
  // covering each block fully, covering each 16x16 region fully
  uint32_t mask4[CV_WORDS][64], mask4f[CV_WORDS][64], mask16[CV_WORDS][4];
  // the round's pairs: per block up to CV_K staged-triangle indices (bit 7:
  // the block is covered fully), their count, the blocks' offsets into the
  // dense pair numbering, and each pair's coverage (uncut, cut to the
  // target; quad-major, so quad q's 16 bits are its 16-bit word q)
  uint8_t slot[64][CV_K];
  uint32_t off[64], wtot[CV_THREADS / 32];
  unsigned long long cov_uc[64][CV_K], cov_cv[64][CV_K];
  float spx[4], spy[4];
  uint32_t item;
  // the batch's bin entries, and the fill's per-warp counts and resume point
  uint32_t cand[CV_STAGE];
  uint32_t wcnt[CV_THREADS / 32];
  uint32_t next;
  // the walk: each quad's fragment list cursor, the quads with covered
  // pairs in the round (quad << 16 | pair bits), packed, and per block
  // whether a walk wrote depth since its range was last taken
  uint32_t own_first[CV_THREADS], own_cur[CV_THREADS], own_count[CV_THREADS];
  uint32_t walk[CV_THREADS];
  uint32_t nwalk;
  uint32_t keycnt[128];  // fragments per shade key (cover_counts_classes)
  uint8_t zdirty[64];
};
// followed by the staged depth: CV_PX * CV_PX * samples words (early-Z only)
inline size_t cv_smem(uint32_t samples, bool early_z) {
  return ((sizeof(CvShared) + 15) & ~size_t(15)) + (early_z ? static_cast<size_t>(CV_PX) * CV_PX * samples * 4 : 0);
}

// This thread's quad: pixel i at (x + (i & 1), y + (i >> 1)).
struct Quad {
  int x, y;         // target coordinates of its top-left pixel
  uint32_t inside;  // bit i: pixel i inside the target
  uint32_t samples;
  float ax[4], ay[4];  // offsets of the samples from the pixel centre (aa_z_offset)
};

// Depth range stored in a quad or block (pixels inside the target only).
struct ZRange {
  float zmax, zmin;
  uint32_t qmax, qmin;  // D24 depth bits
};

__device__ inline void z_range(uint32_t const* zq, int zrow, Quad const& qd, bool d24, ZRange& r) {
  uint32_t const S = qd.samples;
  r.zmax = -INFINITY;
  r.zmin = INFINITY;
  r.qmax = 0;
  r.qmin = 0xFFFFFFu;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (!((qd.inside >> i) & 1u)) continue;
    uint32_t const* zp = zq + (i >> 1) * zrow + (i & 1) * S;
    if (S == 4) {  // the pixel's four words are one 16-byte word
      uint4 const w4 = *reinterpret_cast<uint4 const*>(zp);
      uint32_t const w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        if (d24) {
          r.qmax = max(r.qmax, w[s] & 0xFFFFFFu);
          r.qmin = min(r.qmin, w[s] & 0xFFFFFFu);
        } else {
          r.zmax = fmaxf(r.zmax, __uint_as_float(w[s]));
          r.zmin = fminf(r.zmin, __uint_as_float(w[s]));
        }
      }
      continue;
    }
    for (uint32_t s = 0; s < S; ++s) {
      uint32_t w = zp[s];
      if (d24) {
        r.qmax = max(r.qmax, w & 0xFFFFFFu);
        r.qmin = min(r.qmin, w & 0xFFFFFFu);
      } else {
        r.zmax = fmaxf(r.zmax, __uint_as_float(w));
        r.zmin = fminf(r.zmin, __uint_as_float(w));
      }
    }
  }
}

// Whether every sample of the 4x4 block at (bx_abs, by_abs) fails `func` against the
// stored range.
__device__ inline bool z_culled(TriCv const& t, int bx_abs, int by_abs, uint32_t func, bool d24, ZRange const& r) {
  if (func == SG_CMP_NEVER) return true;
  if (func != SG_CMP_LESS && func != SG_CMP_LESS_EQUAL && func != SG_CMP_GREATER && func != SG_CMP_GREATER_EQUAL)
    return false;
  // the depth plane over the block's rectangle; sample positions lie inside it
  float const x0 = static_cast<float>(bx_abs) - t.p0x, x1 = x0 + 4.0f;
  float const y0 = static_cast<float>(by_abs) - t.p0y, y1 = y0 + 4.0f;
  float const ax = t.dzx * x0, bx = t.dzx * x1, ay = t.dzy * y0, by = t.dzy * y1;
  float const lo = t.p0z + (fminf(ax, bx) + fminf(ay, by));
  float const hi = t.p0z + (fmaxf(ax, bx) + fmaxf(ay, by));
  // rounding of the reference's expression and of this bound: well under
  // 2^-19 of the magnitudes involved
  float const mag = fabsf(t.p0z) + fmaxf(fabsf(ax), fabsf(bx)) + fmaxf(fabsf(ay), fabsf(by)) +
                    2.0f * (fabsf(t.dzx) + fabsf(t.dzy));
  float const margin = mag * 1.9073486328125e-06f + 1e-30f;
  float const L = lo - margin, U = hi + margin;
  if (d24) {
    uint32_t const lq = d24_quantize(L), uq = d24_quantize(U);
    switch (func) {
    case SG_CMP_LESS: return lq >= r.qmax;
    case SG_CMP_LESS_EQUAL: return lq > r.qmax;
    case SG_CMP_GREATER: return uq <= r.qmin;
    default: return uq < r.qmin;
    }
  }
  switch (func) {
  case SG_CMP_LESS: return L >= r.zmax;
  case SG_CMP_LESS_EQUAL: return L > r.zmax;
  case SG_CMP_GREATER: return U <= r.zmin;
  default: return U < r.zmin;
  }
}

// Whether the hierarchical depth test drops the pair on the block at (bx, by).
__device__ inline bool pair_hidden(TriCv const& t, int bx, int by, bool d24, ZRange const& zr) {
  uint32_t const zc = t.zcfg, func = (zc >> 8) & 15u;
  return (zc & 128u) && (((zc >> 4) & 1u) || func == SG_CMP_NEVER) && z_culled(t, bx, by, func, d24, zr);
}

// Nibble of block pixel (ix, iy) in a quad-major block mask: quad
// q = (iy / 2) * 2 + ix / 2, then pixel i = (iy % 2) * 2 + ix % 2 of the quad.
__host__ __device__ constexpr int qnib(int ix, int iy) { return ((iy >> 1) * 2 + (ix >> 1)) * 4 + (iy & 1) * 2 + (ix & 1); }

// Per-sample coverage of a whole 4x4 block (draw_partial_tile's edge test,
// rasterizer.cpp:298-439): 4 bits (samples) per pixel, pixel (ix, iy) at
// nibble qnib(ix, iy); `uc` uncut, `cv` cut to the pixels inside the target
// (`inside`: bit qnib(ix, iy)).
__device__ inline void block_coverage(TriCv const& t, bool full, int bx_abs, int by_abs, uint32_t S, float const* spx,
                                      float const* spy, uint32_t inside, uint64_t& uc, uint64_t& cv) {
  uc = 0;
  if (full) {
    uint64_t fm = (1ull << S) - 1ull;
#pragma unroll
    for (int p = 0; p < 16; ++p) uc |= fm << (4 * p);
  } else {
    float4 const e[3] = {t.e0, t.e1, t.e2};
    float const lf = static_cast<float>(bx_abs), tf = static_cast<float>(by_abs);
    float ev[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) ev[k] = e[k].z - (lf * e[k].x + tf * e[k].y);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      if (s >= static_cast<int>(S)) break;
      float const sx = spx[s], sy = spy[s];
#pragma unroll
      for (int iy = 0; iy < 4; ++iy) {
        float const my = sy + static_cast<float>(iy);
#pragma unroll
        for (int ix = 0; ix < 4; ++ix) {
          float const mx = sx + static_cast<float>(ix);
          bool rej = false;
#pragma unroll
          for (int k = 0; k < 3; ++k) rej = rej || ((mx * e[k].x + my * e[k].y) < ev[k]);
          uc |= static_cast<uint64_t>(!rej) << (qnib(ix, iy) * 4 + s);
        }
      }
    }
  }
  // EXTENSION: pixels outside the target are not covered
  uint64_t im = 0;
#pragma unroll
  for (int p = 0; p < 16; ++p)
    if ((inside >> p) & 1u) im |= 0xFull << (4 * p);
  cv = uc & im;
}

// Quad q's 16 coverage bits (4 per pixel i, in quad order) of a quad-major
// block mask in shared memory.
__device__ inline uint32_t quad_bits(unsigned long long const& m, int q) {
  return reinterpret_cast<uint16_t const*>(&m)[q];
}

// Early-Z of one pair on this thread's quad (framebuffer.cpp:522-614)
// against the staged depth: returns the passing samples of the covered ones
// `cq` and writes depth on pass.
// FUNC: the depth function when known at compile time (LESS or LESS_EQUAL,
// which read depth), else -1 and it and the depth format are read from
// the draw's configuration per sample.
template <int FUNC, bool D24>
__device__ inline uint32_t early_z_quad(TriCv const& t, uint32_t cq, uint32_t* zq, int zrow, Quad const& qd,
                                        bool& wrote) {
  uint32_t const S = qd.samples, zc = t.zcfg, func = (zc >> 8) & 15u;
  bool const rd = (zc >> 4) & 1u, wr = (zc >> 5) & 1u, d24 = FUNC < 0 ? ((zc >> 6) & 1u) != 0 : D24;
  // step_2d_unproj_pos_quad's z (shader.cpp:257-287)
  float const dx = 0.5f + static_cast<float>(qd.x) - t.p0x;
  float const dy = 0.5f + static_cast<float>(qd.y) - t.p0y;
  float const z00 = t.p0z + (t.dzx * dx + t.dzy * dy);
  uint32_t tz = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint32_t const pbits = (cq >> (4 * i)) & 0xFu;
    if (!pbits) continue;
    float const z = (i & 2) ? ((i & 1) ? (z00 + t.dzx) + t.dzy : z00 + t.dzy) : ((i & 1) ? z00 + t.dzx : z00);
    uint32_t* zp = zq + (i >> 1) * zrow + (i & 1) * S;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      if (!(pbits & (1u << s))) continue;  // coverage holds samples below S only
      float const nd = S == 1 ? z : (qd.ax[s] * t.dzx + qd.ay[s] * t.dzy) + z;
      uint32_t const w = zp[s];
      bool pass;
      if constexpr (FUNC == SG_CMP_LESS)
        pass = D24 ? d24_quantize(nd) < (w & 0xFFFFFFu) : nd < __uint_as_float(w);
      else if constexpr (FUNC == SG_CMP_LESS_EQUAL)
        pass = D24 ? d24_quantize(nd) <= (w & 0xFFFFFFu) : nd <= __uint_as_float(w);
      else
        pass = d24 ? cmpu(func, d24_quantize(nd), rd ? (w & 0xFFFFFFu) : 0u)
                   : cmpf(func, nd, rd ? __uint_as_float(w) : 0.0f);
      if (pass) {
        if (wr) {
          zp[s] = d24 ? ((w & 0xFF000000u) | d24_quantize(nd)) : __float_as_uint(nd);
          wrote = true;
        }
        tz |= 1u << (4 * i + s);
      }
    }
  }
  return tz;
}

// early_z_quad for four samples and a compiled LESS / LESS_EQUAL: a pixel's
// four depth words are one 16-byte word of the staged depth, read once,
// tested sample by sample without branches and written once.  The sample
// depth is the same expression as early_z_quad's, in the same order.
template <int FUNC, bool D24>
__device__ inline uint32_t early_z_quad4(TriCv const& t, uint32_t cq, uint32_t* zq, int zrow, Quad const& qd,
                                         bool& wrote) {
  bool const wr = (t.zcfg >> 5) & 1u;
  float const dx = 0.5f + static_cast<float>(qd.x) - t.p0x;
  float const dy = 0.5f + static_cast<float>(qd.y) - t.p0y;
  float const z00 = t.p0z + (t.dzx * dx + t.dzy * dy);
  float off[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) off[s] = qd.ax[s] * t.dzx + qd.ay[s] * t.dzy;
  uint32_t tz = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint32_t const pbits = (cq >> (4 * i)) & 0xFu;
    if (!pbits) continue;
    float const z = (i & 2) ? ((i & 1) ? (z00 + t.dzx) + t.dzy : z00 + t.dzy) : ((i & 1) ? z00 + t.dzx : z00);
    uint4* const zp = reinterpret_cast<uint4*>(zq + (i >> 1) * zrow + (i & 1) * 4);
    uint4 const w4 = *zp;
    uint32_t w[4] = {w4.x, w4.y, w4.z, w4.w};
    uint32_t pass = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      float const nd = off[s] + z;
      uint32_t const q24 = D24 ? d24_quantize(nd) : 0u;
      bool p;
      if constexpr (FUNC == SG_CMP_LESS)
        p = D24 ? q24 < (w[s] & 0xFFFFFFu) : nd < __uint_as_float(w[s]);
      else
        p = D24 ? q24 <= (w[s] & 0xFFFFFFu) : nd <= __uint_as_float(w[s]);
      p = p && ((pbits >> s) & 1u);
      pass |= static_cast<uint32_t>(p) << s;
      uint32_t const nw = D24 ? ((w[s] & 0xFF000000u) | q24) : __float_as_uint(nd);
      w[s] = p ? nw : w[s];
    }
    if (pass && wr) {
      *zp = make_uint4(w[0], w[1], w[2], w[3]);
      wrote = true;
    }
    tz |= pass << (4 * i);
  }
  return tz;
}

// Fills the batch: from bin entry `bpos` on, the entries whose triangle's
// bounding box reaches the quadrant (x in [qx0, qx0 + 32), y in [qy0,
// qy0 + 32) of the tile), in order, at most CV_STAGE of them.  A triangle
// whose box misses the quadrant misses every one of its regions, so the
// classification below would give it no bit.  Returns the batch's size and
// advances `bpos` past the last entry taken (or examined).
__device__ inline uint32_t cv_fill(PassParams const& P, uint32_t& bpos, uint32_t end, int tile_x0, int tile_y0,
                                   int qx0, int qy0, CvShared& sh) {
  float const tx0f = static_cast<float>(tile_x0), ty0f = static_cast<float>(tile_y0);
  float const xs = static_cast<float>(qx0), xe = xs + CV_PX, ys = static_cast<float>(qy0), ye = ys + CV_PX;
  int const tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t nst = 0;
  for (;;) {
    uint32_t const cand = bpos + tid;
    uint32_t e = 0;
    bool reach = false;
    if (cand < end) {
      e = P.bin_entries[cand];
      reach = (e & 1u) != 0;  // accepted for the whole tile by the binner
      if (!reach) {
        float4 const bb = P.recs[(e >> 1) + 3];
        reach = !(bb.x - tx0f >= xe || bb.y - tx0f < xs || bb.z - ty0f >= ye || bb.w - ty0f < ys);
      }
    }
    uint32_t const bal = __ballot_sync(0xFFFFFFFFu, reach);
    if (lane == 0) sh.wcnt[warp] = __popc(bal);
    __syncthreads();
    uint32_t excl = __popc(bal & ((1u << lane) - 1u)), total = 0;
#pragma unroll
    for (int w = 0; w < CV_THREADS / 32; ++w) {
      uint32_t const c = sh.wcnt[w];
      excl += w < warp ? c : 0u;
      total += c;
    }
    uint32_t const room = CV_STAGE - nst;
    if (reach && excl < room) sh.cand[nst + excl] = e;
    if (reach && excl == room) sh.next = cand;
    __syncthreads();
    if (total > room) {
      bpos = sh.next;
      return CV_STAGE;
    }
    nst += total;
    bpos = min(bpos + CV_THREADS, end);
    if (nst == CV_STAGE || bpos >= end) return nst;
  }
}

// Stages the batch's triangles and classifies each against the quadrant's
// regions and blocks (rasterizer.cpp:441-571); two threads per triangle, one
// per row of 16x16 regions.
__device__ inline void cv_stage(PassParams const& P, TargetParams const& T, uint32_t nb, int tile_x0, int tile_y0,
                                int bx0, int by0, CvShared& sh) {
  float const tx0f = static_cast<float>(tile_x0), ty0f = static_cast<float>(tile_y0);
  float const trr = T.target_w, trb = T.target_h;
  for (uint32_t j = threadIdx.x; j < 2 * nb; j += CV_THREADS) {
    uint32_t const i = j >> 1, row = j & 1;
    uint32_t const e = sh.cand[i];
    float4 const* R = P.recs + (e >> 1);
    TriCv ts;
    ts.e0 = R[0];
    ts.e1 = R[1];
    ts.e2 = R[2];
    ts.bbox = R[3];
    float4 const r4 = R[4];
    ts.p0x = ts.e0.w;
    ts.p0y = ts.e1.w;
    ts.p0z = ts.e2.w;
    ts.dzx = r4.x;
    ts.dzy = r4.y;
    ts.entry = e;
    uint32_t const flags = __float_as_uint(r4.w);
    ts.zcfg = flags & 0x1FFFu;
    ts.shade_key = (flags >> 24) & 127u;
    if (row == 0) sh.stage[i] = ts;
    uint32_t const bit = 1u << (i & 31), word = i >> 5;
    if (e & 1u) {  // accepted for the whole tile by the binner
      atomicOr(&sh.mask16[word][2 * row], bit);
      atomicOr(&sh.mask16[word][2 * row + 1], bit);
      continue;
    }
    float const x_min = ts.bbox.x - tx0f, x_max = ts.bbox.y - tx0f, y_min = ts.bbox.z - ty0f,
                y_max = ts.bbox.w - ty0f;
    float4 const ed[3] = {ts.e0, ts.e1, ts.e2};
    LevelParams l1, l2;
    level_params(ed, l1, l2);
    // blocks (tile numbering) the bounding box can reach; the exact
    // reference tests below decide
    int const jx_lo = max(bx0, static_cast<int>(floorf(x_min * 0.25f)) - 1);
    int const jx_hi = min(bx0 + 7, static_cast<int>(floorf(x_max * 0.25f)) + 1);
    int const jy_lo = max(by0, static_cast<int>(floorf(y_min * 0.25f)) - 1);
    int const jy_hi = min(by0 + 7, static_cast<int>(floorf(y_max * 0.25f)) + 1);
    {
      int const iy = (by0 >> 2) + static_cast<int>(row);
      int const m16y = iy * 16;
      if (y_min >= static_cast<float>(m16y + 16) || y_max < static_cast<float>(m16y)) continue;
      for (int ix = bx0 >> 2; ix < (bx0 >> 2) + 2; ++ix) {
        int const m16x = ix * 16;
        if (x_min >= static_cast<float>(m16x + 16) || x_max < static_cast<float>(m16x)) continue;
        int const c = child_class(ed, l1, tx0f, ty0f, ix, iy);
        if (c == 0) continue;
        // a region whose origin is right of / below the target is skipped
        if (static_cast<float>(tile_x0 + m16x) >= trr || static_cast<float>(tile_y0 + m16y) >= trb) continue;
        int const r = (iy - (by0 >> 2)) * 2 + (ix - (bx0 >> 2));
        if (c == 2) {
          atomicOr(&sh.mask16[word][r], bit);
          continue;
        }
        // partial: level 2 over the 4x4 children inside the bounding box
        float const r16xf = static_cast<float>(tile_x0 + m16x), r16yf = static_cast<float>(tile_y0 + m16y);
        for (int jy = max(0, jy_lo - iy * 4); jy <= min(3, jy_hi - iy * 4); ++jy) {
          int const m4y = m16y + jy * 4;
          if (y_min >= static_cast<float>(m4y + 4) || y_max < static_cast<float>(m4y)) continue;
          if (static_cast<float>(tile_y0 + m4y) >= trb) continue;
          for (int jx = max(0, jx_lo - ix * 4); jx <= min(3, jx_hi - ix * 4); ++jx) {
            int const m4x = m16x + jx * 4;
            if (x_min >= static_cast<float>(m4x + 4) || x_max < static_cast<float>(m4x)) continue;
            if (static_cast<float>(tile_x0 + m4x) >= trr) continue;
            int const c2 = child_class(ed, l2, r16xf, r16yf, jx, jy);
            if (c2 == 0) continue;
            int const bi = (iy * 4 + jy - by0) * 8 + (ix * 4 + jx - bx0);
            atomicOr(&sh.mask4[word][bi], bit);
            if (c2 == 2) atomicOr(&sh.mask4f[word][bi], bit);
          }
        }
      }
    }
  }
}

// MINB: CTAs per SM the register budget is cut for (3: 80 registers, 4: 64)
template <int MINB>
__global__ void __launch_bounds__(CV_THREADS, MINB) k_cover2(PassParams P) {
  pdl_wait();
  extern __shared__ __align__(16) uint8_t smem_raw[];
  CvShared& sh = *reinterpret_cast<CvShared*>(smem_raw);
  uint32_t* const ztile = reinterpret_cast<uint32_t*>(smem_raw + ((sizeof(CvShared) + 15) & ~size_t(15)));
  if ((P.counters->overflow & (OVF_BIN | OVF_REC)) || pass_gated(P)) return;
  // item block ib = 0..63 at (ib & 7, ib >> 3); this thread's quad q of it
  // has its top-left pixel at block pixel (qx0, qy0)
  int const tid = threadIdx.x, q = tid & 3, ib = tid >> 2;
  int const ibx = ib & 7, iby = ib >> 3, qx0 = (q & 1) * 2, qy0 = (q >> 1) * 2;
  uint32_t const nitems = P.ntiles * 4;
  if (tid < 128) sh.keycnt[tid] = 0;  // ordered before use by the item loop's first barrier
  for (;;) {
    if (tid == 0) sh.item = atomicAdd(&P.counters->tile_cursor, 1u);
    __syncthreads();
    uint32_t const item = sh.item;
    __syncthreads();
    if (item >= nitems) break;
    uint32_t const tile = P.tile_order ? P.tile_order[item >> 2] : item >> 2, sub = item & 3;
    uint32_t const begin = P.tile_begin[tile], end = P.tile_begin[tile + 1];
    TargetParams const& T = P.targets[target_of_tile(P, tile)];
    uint32_t const ltile = tile - T.tile_base;
    int const tile_x0 = static_cast<int>(ltile % T.tiles_x) * TILE, tile_y0 = static_cast<int>(ltile / T.tiles_x) * TILE;
    int const bx0 = (sub & 1) * 8, by0 = (sub >> 1) * 8;  // first block of the quadrant, tile numbering
    int const x0 = tile_x0 + bx0 * 4, y0 = tile_y0 + by0 * 4;
    uint32_t const S = T.samples, W = T.width, H = T.height;
    if (tid < 4) {
      sh.spx[tid] = T.sp_x[tid];
      sh.spy[tid] = T.sp_y[tid];
    }
    int const bx = bx0 + ibx, by = by0 + iby;  // this thread's block, tile numbering
    int const own16 = (iby >> 2) * 2 + (ibx >> 2);  // its 16x16 region within the quadrant
    sh.own_first[tid] = sh.own_cur[tid] = NO_CHUNK;
    sh.own_count[tid] = 0;
    if (q == 0) sh.zdirty[ib] = 0;
    Quad qd;
    qd.x = tile_x0 + bx * 4 + qx0;
    qd.y = tile_y0 + by * 4 + qy0;
    qd.samples = S;
#pragma unroll
    for (uint32_t s = 0; s < 4; ++s) {
      uint32_t const sm = min(s, S - 1);
      qd.ax[s] = T.sp_x[sm] - 0.5f;
      qd.ay[s] = T.sp_y[sm] - 0.5f;
    }
    qd.inside = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (static_cast<uint32_t>(qd.x + (i & 1)) < W && static_cast<uint32_t>(qd.y + (i >> 1)) < H) qd.inside |= 1u << i;
    bool const stage_z = T.any_early_z && begin < end;
    bool const d24 = T.ds_fmt == SG_FMT_D24S8;
    uint32_t const qw = min(static_cast<uint32_t>(CV_PX), W - min(W, static_cast<uint32_t>(x0)));
    uint32_t const qh = min(static_cast<uint32_t>(CV_PX), H - min(H, static_cast<uint32_t>(y0)));
    uint32_t const zrow = CV_PX * S;
    if (stage_z) {
      // the quadrant's depth, and its pre-image for k_cover_rollback
      uint32_t* const zb = (P.zbackup && !T.zpre_known) ? P.zbackup + static_cast<size_t>(tile) * P.zbackup_tile_words +
                                           (static_cast<size_t>(by0) * 4 * TILE + bx0 * 4) * S
                                     : nullptr;
#pragma unroll 4
      for (uint32_t i = tid; i < qh * zrow; i += CV_THREADS) {
        uint32_t y = i >> (__ffs(zrow) - 1), k = i & (zrow - 1);  // zrow: a power of two
        if (k >= qw * S) continue;
        uint32_t x = k >> (S >> 1), sm = k & (S - 1);
        uint32_t const v = *reinterpret_cast<uint32_t const*>(ds_addr(T, x0 + x, y0 + y, sm));
        ztile[i] = v;
        if (zb) zb[static_cast<size_t>(y) * TILE * S + k] = v;
      }
    }
    uint32_t* const zq = ztile + (iby * 4 + qy0) * zrow + (ibx * 4 + qx0) * S;
    ZRange zr{-INFINITY, INFINITY, 0u, 0xFFFFFFu};  // the block's
    bool z_dirty = stage_z;  // the depth range is recomputed before a batch's culling when stale
    __syncthreads();
    for (uint32_t bpos = begin; bpos < end;) {
      z_dirty = z_dirty || sh.zdirty[ib] != 0;
      if (__any_sync(0xFFFFFFFFu, z_dirty)) {  // the block's range: its four quads' ranges combined
        z_range(zq, static_cast<int>(zrow), qd, d24, zr);
#pragma unroll
        for (int o = 1; o < 4; o <<= 1) {
          zr.zmax = fmaxf(zr.zmax, __shfl_xor_sync(0xFFFFFFFFu, zr.zmax, o));
          zr.zmin = fminf(zr.zmin, __shfl_xor_sync(0xFFFFFFFFu, zr.zmin, o));
          zr.qmax = max(zr.qmax, __shfl_xor_sync(0xFFFFFFFFu, zr.qmax, o));
          zr.qmin = min(zr.qmin, __shfl_xor_sync(0xFFFFFFFFu, zr.qmin, o));
        }
        z_dirty = false;
      }
      __syncthreads();
      if (q == 0) sh.zdirty[ib] = 0;
      uint32_t* const masks = &sh.mask4[0][0];
      for (int i = tid; i < (64 + 64 + 4) * CV_WORDS; i += CV_THREADS) masks[i] = 0;
      uint32_t const nb = cv_fill(P, bpos, end, tile_x0, tile_y0, bx0 * 4, by0 * 4, sh);
      if (nb == 0) break;
      if (tid == 0) atomicAdd(&P.counters->cover_batches, 1u);
      cv_stage(P, T, nb, tile_x0, tile_y0, bx0, by0, sh);
      __syncthreads();
      // the block's triangles without the hidden ones; the block's four
      // threads test every fourth triangle each
      uint32_t live[CV_WORDS];
#pragma unroll
      for (int w = 0; w < CV_WORDS; ++w) {
        uint32_t const m = sh.mask4[w][ib] | sh.mask16[w][own16];
        uint32_t hid = 0;
        if (stage_z) {
          uint32_t scan = m & (0x11111111u << q);
          while (scan) {
            int const b = __ffs(scan) - 1;
            scan &= scan - 1;
            if (pair_hidden(sh.stage[(w << 5) + b], qd.x - qx0, qd.y - qy0, d24, zr)) hid |= 1u << b;
          }
          hid |= __shfl_xor_sync(0xFFFFFFFFu, hid, 1);
          hid |= __shfl_xor_sync(0xFFFFFFFFu, hid, 2);
        }
        live[w] = m & ~hid;
      }
      for (;;) {
        // this round's pairs: the block's next CV_K triangles in primitive order
        uint32_t n = 0;
        if (tid == 0) sh.nwalk = 0;
#pragma unroll
        for (int w = 0; w < CV_WORDS; ++w) {
          uint32_t const fulls = sh.mask4f[w][ib] | sh.mask16[w][own16];
          while (live[w] && n < static_cast<uint32_t>(CV_K)) {
            int const b = __ffs(live[w]) - 1;
            live[w] &= live[w] - 1;
            if (q == 0) sh.slot[ib][n] = static_cast<uint8_t>((w << 5) + b) | static_cast<uint8_t>(((fulls >> b) & 1u) << 7);
            ++n;
          }
        }
        bool more = false;
#pragma unroll
        for (int w = 0; w < CV_WORDS; ++w) more = more || live[w] != 0;
        {  // the blocks' offsets in the dense pair numbering: within each warp
           // (its eight blocks) by a shuffle scan, across warps by their totals
          uint32_t const lane = tid & 31, v = q == 0 ? n : 0u;
          uint32_t incl = v;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            uint32_t const y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += y;
          }
          if (q == 0) sh.off[ib] = incl - v;  // warp-local
          if (lane == 31) sh.wtot[tid >> 5] = incl;
        }
        __syncthreads();
        // coverage of every pair of the round, spread over all threads
        uint32_t total = 0;
#pragma unroll
        for (int w = 0; w < CV_THREADS / 32; ++w) total += sh.wtot[w];
        if (tid == 0) {
          atomicAdd(&P.counters->cover_rounds, 1u);
          atomicAdd(&P.counters->cover_pairs, total);
        }
        for (uint32_t d = tid; d < total; d += CV_THREADS) {
          uint32_t w = 0, base = 0;
          for (;;) {  // the warp whose blocks hold pair d (d < total: one does)
            uint32_t const t = sh.wtot[w];
            if (d < base + t || w + 1 == CV_THREADS / 32) break;
            base += t;
            ++w;
          }
          uint32_t const dl = d - base;
          uint32_t const b = w * 8 + upper_index(sh.off + w * 8, 8, dl), k = dl - sh.off[b];
          uint32_t const e8 = sh.slot[b][k];
          int const pbx = tile_x0 + (bx0 + static_cast<int>(b & 7)) * 4;
          int const pby = tile_y0 + (by0 + static_cast<int>(b >> 3)) * 4;
          uint32_t inside = 0;
          for (int iy = 0; iy < 4; ++iy)
            for (int ix = 0; ix < 4; ++ix)
              if (static_cast<uint32_t>(pbx + ix) < W && static_cast<uint32_t>(pby + iy) < H) inside |= 1u << qnib(ix, iy);
          uint64_t uc, cv;
          block_coverage(sh.stage[e8 & 127u], (e8 >> 7) != 0, pbx, pby, S, sh.spx, sh.spy, inside, uc, cv);
          sh.cov_uc[b][k] = uc;
          sh.cov_cv[b][k] = cv;
        }
        __syncthreads();
        // the block's pairs in primitive order on each quad: early-Z, then the
        // surviving quad into the quad's fragment list.  The quads with a
        // covered pair this round are packed onto the first threads (any
        // thread walks any quad: its list cursor is in shared memory), so
        // the walk runs on as few, as full warps as the round allows.
        {
          uint32_t covb = 0;
          for (uint32_t k = 0; k < n; ++k) covb |= (quad_bits(sh.cov_cv[ib][k], q) != 0u ? 1u : 0u) << k;
          uint32_t const lane = tid & 31;
          uint32_t const bal = __ballot_sync(0xFFFFFFFFu, covb != 0u);
          uint32_t wbase = 0;  // the warp's walkers take consecutive slots
          if (lane == 0 && bal) wbase = atomicAdd(&sh.nwalk, static_cast<uint32_t>(__popc(bal)));
          wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0);
          if (covb) sh.walk[wbase + __popc(bal & ((1u << lane) - 1u))] = (static_cast<uint32_t>(tid) << 16) | covb;
          __syncthreads();
          uint32_t const nwalk = sh.nwalk;
          if (static_cast<uint32_t>(tid) < nwalk) {
            uint32_t const wk = sh.walk[tid], h = wk >> 16, hq = h & 3u, hb = h >> 2;
            uint32_t pend = wk & 0xFFFFu;
            // the walked quad
            Quad qw;
            qw.x = tile_x0 + (bx0 + static_cast<int>(hb & 7u)) * 4 + static_cast<int>(hq & 1u) * 2;
            qw.y = tile_y0 + (by0 + static_cast<int>(hb >> 3)) * 4 + static_cast<int>(hq >> 1) * 2;
            qw.samples = S;
#pragma unroll
            for (uint32_t sm = 0; sm < 4; ++sm) {
              qw.ax[sm] = sh.spx[min(sm, S - 1)] - 0.5f;
              qw.ay[sm] = sh.spy[min(sm, S - 1)] - 0.5f;
            }
            qw.inside = 0;
#pragma unroll
            for (int i = 0; i < 4; ++i)
              if (static_cast<uint32_t>(qw.x + (i & 1)) < W && static_cast<uint32_t>(qw.y + (i >> 1)) < H)
                qw.inside |= 1u << i;
            uint32_t* const zqw = ztile + ((hb >> 3) * 4 + (hq >> 1) * 2) * zrow + ((hb & 7u) * 4 + (hq & 1u) * 2) * S;
            OwnerList Lw{sh.own_first[h], sh.own_cur[h], sh.own_count[h]};
            uint32_t const fm = (1u << S) - 1u, qfull = fm | (fm << 4) | (fm << 8) | (fm << 12);
            bool wrote_any = false;
            while (pend) {
              uint32_t const k = static_cast<uint32_t>(__ffs(pend) - 1);
              pend &= pend - 1u;
              uint32_t const e8 = sh.slot[hb][k], idx = e8 & 127u;
              uint32_t const cq = quad_bits(sh.cov_cv[hb][k], static_cast<int>(hq));
              TriCv const& t = sh.stage[idx];
              uint32_t tq = cq;
              if (t.zcfg & 128u) {
                bool wrote = false;
                // the common depth functions with the compare as code, not data
                uint32_t const zc = t.zcfg, func = (zc >> 8) & 15u;
                bool const d24z = (zc >> 6) & 1u;
                int const zr_ = static_cast<int>(zrow);
                if (S == 4 && func == SG_CMP_LESS)
                  tq = d24z ? early_z_quad4<SG_CMP_LESS, true>(t, cq, zqw, zr_, qw, wrote)
                            : early_z_quad4<SG_CMP_LESS, false>(t, cq, zqw, zr_, qw, wrote);
                else if (S == 4 && func == SG_CMP_LESS_EQUAL)
                  tq = d24z ? early_z_quad4<SG_CMP_LESS_EQUAL, true>(t, cq, zqw, zr_, qw, wrote)
                            : early_z_quad4<SG_CMP_LESS_EQUAL, false>(t, cq, zqw, zr_, qw, wrote);
                else if (func == SG_CMP_LESS)
                  tq = d24z ? early_z_quad<SG_CMP_LESS, true>(t, cq, zqw, zr_, qw, wrote)
                            : early_z_quad<SG_CMP_LESS, false>(t, cq, zqw, zr_, qw, wrote);
                else if (func == SG_CMP_LESS_EQUAL)
                  tq = d24z ? early_z_quad<SG_CMP_LESS_EQUAL, true>(t, cq, zqw, zr_, qw, wrote)
                            : early_z_quad<SG_CMP_LESS_EQUAL, false>(t, cq, zqw, zr_, qw, wrote);
                else
                  tq = early_z_quad<-1, false>(t, cq, zqw, zr_, qw, wrote);
                wrote_any = wrote_any || wrote;
              }
              if (!tq) continue;
              uint32_t const uq = quad_bits(sh.cov_uc[hb][k], static_cast<int>(hq));
              bool const fullq = (e8 >> 7) ? cq == qfull : (uq == qfull && cq == uq);
              if (owner_append(P, Lw, t.entry >> 1,
                               (static_cast<uint32_t>(qw.x) >> 1) | ((static_cast<uint32_t>(qw.y) >> 1) << 12) |
                                   (fullq ? 1u << 24 : 0u) | (t.shade_key << 25),
                               tq | (cq << 16)) &&
                  P.cover_counts_classes)
                atomicAdd(&sh.keycnt[t.shade_key], 1u);
            }
            sh.own_first[h] = Lw.first;
            sh.own_cur[h] = Lw.cur;
            sh.own_count[h] = Lw.count;
            if (wrote_any) sh.zdirty[hb] = 1;
          }
        }
        if (!__syncthreads_or(more)) break;
      }
    }
    if (stage_z) {
      __syncthreads();
      for (uint32_t i = tid; i < qh * zrow; i += CV_THREADS) {
        uint32_t y = i >> (__ffs(zrow) - 1), k = i & (zrow - 1);  // zrow: a power of two
        if (k >= qw * S) continue;
        uint32_t x = k >> (S >> 1), sm = k & (S - 1);
        *reinterpret_cast<uint32_t*>(ds_addr(T, x0 + x, y0 + y, sm)) = ztile[i];
      }
    }
    // close the quad's list for the item
    __syncthreads();
    uint32_t const lcur = sh.own_cur[tid];
    if (lcur != NO_CHUNK) {
      P.chunk_next[lcur] = NO_CHUNK;
      P.chunk_count[lcur] = sh.own_count[tid];
    }
    P.owner_first[static_cast<size_t>(tile) * QUAD_OWNERS + (by * 2 + (q >> 1)) * 32 + bx * 2 + (q & 1)] =
        sh.own_first[tid];
  }
  if (P.cover_counts_classes) {  // the CTA's fragments per shade key, once
    __syncthreads();
    if (tid < 128 && sh.keycnt[tid]) atomicAdd(&P.class_counts[tid], sh.keycnt[tid]);
  }
}

// Undoes the coverage pass's depth write-back when the pass overflowed after
// it (fragments, or the learned filter's lookup queue): every tile the
// coverage pass staged gets its pre-image back from P.zbackup, so the pass
// leaves its targets as it found them and the host can run it again.  (A
// pass that overflowed its bins or records skipped the coverage pass.)
__global__ void __launch_bounds__(256) k_cover_rollback(PassParams P) {
  pdl_wait();
  if (pass_gated(P)) return;
  uint32_t const ovf = P.counters->overflow;
  if (!(ovf & (OVF_FRAG | OVF_AF_QUEUE)) || (ovf & (OVF_BIN | OVF_REC))) return;
  for (uint32_t tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
    if (P.tile_begin[tile] == P.tile_begin[tile + 1]) continue;
    TargetParams const& T = P.targets[target_of_tile(P, tile)];
    if (!T.any_early_z) continue;
    bool const known = T.zpre_known != 0;  // the pass's clear set every depth word
    uint32_t const ltile = tile - T.tile_base, S = T.samples;
    uint32_t const tx0 = (ltile % static_cast<uint32_t>(T.tiles_x)) * TILE;
    uint32_t const ty0 = (ltile / static_cast<uint32_t>(T.tiles_x)) * TILE;
    uint32_t const tw = min(static_cast<uint32_t>(TILE), T.width - min(T.width, tx0));
    uint32_t const th = min(static_cast<uint32_t>(TILE), T.height - min(T.height, ty0));
    uint32_t const* zb = known ? nullptr : P.zbackup + static_cast<size_t>(tile) * P.zbackup_tile_words;
    for (uint32_t i = threadIdx.x; i < th * TILE * S; i += blockDim.x) {
      uint32_t const y = i >> (6 + (S >> 1)), k = i & (TILE * S - 1), x = k >> (S >> 1), sm = k & (S - 1);
      if (x >= tw) continue;
      *reinterpret_cast<uint32_t*>(ds_addr(T, tx0 + x, ty0 + y, sm)) = known ? T.zpre_word : zb[i];
    }
  }
}

// Adds the pass's coverage work counts to the device's profile totals.
__global__ void k_cover_count(PassParams P, unsigned long long* acc) {
  if ((P.counters->overflow & OVF_FATAL) || pass_gated(P)) return;
  acc[2] += P.counters->cover_batches;
  acc[3] += P.counters->cover_rounds;
  acc[4] += P.counters->cover_pairs;
}
void launch_cover_count(PassParams const& p, unsigned long long* acc, cudaStream_t s) {
  k_cover_count<<<1, 1, 0, s>>>(p, acc);
}

void launch_cover_rollback(PassParams const& p, uint32_t grid, cudaStream_t s) {
  launch_pdl(k_cover_rollback, grid, 256, 0, s, p);
}

void launch_cover2(PassParams const& p, uint32_t max_samples, bool early_z, uint32_t ctas_per_sm, uint32_t grid,
                   cudaStream_t s) {
  if (ctas_per_sm >= 4)
    launch_pdl(k_cover2<4>, grid, CV_THREADS, cv_smem(max_samples, early_z), s, p);
  else
    launch_pdl(k_cover2<3>, grid, CV_THREADS, cv_smem(max_samples, early_z), s, p);
}

// Per device (function attributes are per device): the largest dynamic
// shared memory an item needs, and the shared-memory carveout at its
// maximum so that four items' tables fit on an SM.
cudaError_t init_cover2() {
  for (auto fn : {k_cover2<3>, k_cover2<4>}) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(cv_smem(4, true)));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace sg
