// sg_cover.cu -- coverage and early-Z of a pass, two threads per 4x4 block.
//
// Work items are the 32x32 quadrants of every tile of every target, taken
// from a dynamic cursor.  A CTA of 128 threads stages the tile's triangles
// (its bin list, in API order) in batches and classifies each against the
// quadrant's 16x16 regions and 4x4 blocks with the reference's level-1 and
// level-2 trivial reject / accept tests (rasterizer.cpp:441-571), keeping
// per-block sets of the triangles that reach the block and of those that
// cover it fully.  Every block is then walked, in primitive order, by its
// two threads: each tests half of the block's samples (the per-sample edge
// test of draw_partial_tile, rasterizer.cpp:298-439) and runs early-Z on
// them against the quadrant's depth staged in shared memory
// (framebuffer.cpp:522-614).  The pair merges its masks and the block's
// first thread appends the surviving quads to the block's fragment list.
// Samples of one block never depend on each other, so the two threads need
// no ordering beyond walking the same triangle sequence.
//
// Hierarchical depth cull: each thread keeps the largest and smallest depth
// stored in its half of the block.  Before testing a triangle it bounds the
// triangle's depth over the block from the depth plane, widened by a margin
// that covers the rounding of the reference's per-sample depth expression;
// when the bound proves every sample fails the depth test, the pair is
// skipped.  The skipped samples would neither pass nor write, so results are
// those of testing every sample.
#include "sg_raster.cuh"

namespace sg {

constexpr int CV_THREADS = 128;              // 64 blocks x 2 threads
constexpr int CV_STAGE = 128;                // triangles per staged batch
constexpr int CV_WORDS = CV_STAGE / 32;
constexpr int CV_PX = 32;                    // quadrant edge

struct TriCv {  // what coverage and early-Z read of a triangle
  float4 e0, e1, e2, bbox;
  float p0x, p0y, p0z, dzx;
  float dzy;
  uint32_t entry, zcfg, nattr;
};

// shared memory: staged triangles, then per word of the batch the sets
// (one bit per staged triangle): reaching each of the 64 blocks, covering
// each block fully, covering each 16x16 region fully; then the staged depth
constexpr size_t cv_smem_base() {
  return CV_STAGE * sizeof(TriCv) + (64 + 64 + 4) * CV_WORDS * sizeof(uint32_t);
}
size_t cv_smem(uint32_t samples, bool early_z) {
  return cv_smem_base() + (early_z ? static_cast<size_t>(CV_PX) * CV_PX * samples * 4 : 0);
}

// This thread's half of a block: samples [s0, s0 + ns) of rows [r0, r0 + nr).
struct Half {
  uint32_t s0, ns, r0, nr;
  uint32_t inside;  // bit iy * 4 + ix: pixel inside the target
};

// Depth range stored in the thread's half (pixels inside the target only).
struct ZRange {
  float zmax, zmin;
  uint32_t qmax, qmin;  // D24 depth bits
};

__device__ inline void z_range(uint32_t const* zblk, int zrow, uint32_t S, Half const& hf, bool d24, ZRange& r) {
  r.zmax = -INFINITY;
  r.zmin = INFINITY;
  r.qmax = 0;
  r.qmin = 0xFFFFFFu;
  for (uint32_t iy = hf.r0; iy < hf.r0 + hf.nr; ++iy)
#pragma unroll
    for (int ix = 0; ix < 4; ++ix) {
      if (!((hf.inside >> (iy * 4 + ix)) & 1u)) continue;
      uint32_t const* zp = zblk + iy * zrow + ix * S;
      for (uint32_t s = hf.s0; s < hf.s0 + hf.ns; ++s) {
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

// Whether every sample of the block fails `func` against the stored range.
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

// One (triangle, block) pair, half of the block's samples.  `full`: the
// block is covered fully (accepted at level 1 or 2).
__device__ inline void cv_pair(PassParams const& P, TargetParams const& T, TriCv const& t, bool full, int bx_abs,
                               int by_abs, uint32_t* zblk, int zrow, int h, Half const& hf, ZRange& zr,
                               OwnerList& L) {
  uint32_t const S = T.samples;
  uint32_t const zc = t.zcfg;
  bool const early = (zc & 128u) != 0;
  uint32_t const func = (zc >> 8) & 15u;
  bool const rd = (zc >> 4) & 1u, wr = (zc >> 5) & 1u, d24 = (zc >> 6) & 1u;
  // masks over the block, 4 bits (samples) per pixel, pixel (ix, iy) at nibble iy * 4 + ix
  uint64_t uc = 0, cv = 0, tz = 0;
  // (a culled half contributes no coverage bits: exact only where the quads'
  // coverage is not read later, i.e. without centroid interpolation)
  bool const culled = early && !(zc & 4096u) && (rd || func == SG_CMP_NEVER) &&
                      z_culled(t, bx_abs, by_abs, func, d24, zr);
  if (!culled) {
    float4 const e[3] = {t.e0, t.e1, t.e2};
    float const lf = static_cast<float>(bx_abs), tf = static_cast<float>(by_abs);
    float ev[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) ev[k] = e[k].z - (lf * e[k].x + tf * e[k].y);
    for (uint32_t iy = hf.r0; iy < hf.r0 + hf.nr; ++iy) {
      for (uint32_t s = hf.s0; s < hf.s0 + hf.ns; ++s) {
        float const my = T.sp_y[s] + static_cast<float>(iy);
#pragma unroll
        for (int ix = 0; ix < 4; ++ix) {
          bool in = full;
          if (!in) {
            float const mx = T.sp_x[s] + static_cast<float>(ix);
            bool rej = false;
#pragma unroll
            for (int k = 0; k < 3; ++k) rej = rej || ((mx * e[k].x + my * e[k].y) < ev[k]);
            in = !rej;
          }
          if (in) {
            uint64_t bit = 1ull << ((iy * 4 + ix) * 4 + s);
            uc |= bit;
            // EXTENSION: pixels outside the target are not covered
            if ((hf.inside >> (iy * 4 + ix)) & 1u) cv |= bit;
          }
        }
      }
    }
    tz = cv;
    if (early && cv) {  // early-Z: test and write the staged depth now
      tz = 0;
      bool wrote = false;
      for (uint32_t iy = hf.r0; iy < hf.r0 + hf.nr; ++iy) {
        uint32_t const qy = by_abs + (iy & 2u);
        float const dy = 0.5f + static_cast<float>(qy) - t.p0y;
#pragma unroll
        for (int ixq = 0; ixq < 2; ++ixq) {
          uint32_t const qx = bx_abs + 2 * ixq;
          float const dx = 0.5f + static_cast<float>(qx) - t.p0x;
          // step_2d_unproj_pos_quad's z (shader.cpp:257-287)
          float const z00 = t.p0z + (t.dzx * dx + t.dzy * dy);
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            uint32_t const ix = 2 * ixq + i;
            uint32_t const pbits = static_cast<uint32_t>(cv >> ((iy * 4 + ix) * 4)) & 0xFu;
            if (!pbits) continue;
            float const z = (iy & 1u) ? (i ? (z00 + t.dzx) + t.dzy : z00 + t.dzy) : (i ? z00 + t.dzx : z00);
            uint32_t* zp = zblk + iy * zrow + ix * S;
            for (uint32_t s = hf.s0; s < hf.s0 + hf.ns; ++s) {
              if (!(pbits & (1u << s))) continue;
              float const nd = S == 1 ? z : ((T.sp_x[s] - 0.5f) * t.dzx + (T.sp_y[s] - 0.5f) * t.dzy) + z;
              uint32_t const w = zp[s];
              bool const pass = d24 ? cmpu(func, d24_quantize(nd), rd ? (w & 0xFFFFFFu) : 0u)
                                    : cmpf(func, nd, rd ? __uint_as_float(w) : 0.0f);
              if (pass) {
                if (wr) {
                  zp[s] = d24 ? ((w & 0xFF000000u) | d24_quantize(nd)) : __float_as_uint(nd);
                  wrote = true;
                }
                tz |= 1ull << ((iy * 4 + ix) * 4 + s);
              }
            }
          }
        }
      }
      if (wrote) z_range(zblk, zrow, S, hf, d24, zr);
    }
  }
  // merge the halves (the pair walks the same triangles, so both lanes are here)
  uint32_t const lanes = 3u << (threadIdx.x & 30u);
  uc |= __shfl_xor_sync(lanes, uc, 1);
  cv |= __shfl_xor_sync(lanes, cv, 1);
  tz |= __shfl_xor_sync(lanes, tz, 1);
  if (h != 0 || tz == 0) return;
  uint32_t const fm = (1u << S) - 1u;
  uint32_t const qfull = fm | (fm << 4) | (fm << 8) | (fm << 12);
  uint32_t const rec = t.entry >> 1, na = t.nattr << 25;
#pragma unroll 1
  for (int q = 0; q < 4; ++q) {
    int const qx = (q & 1) * 2, qy = (q >> 1) * 2;
    // quad pixel i at (qx + (i & 1), qy + (i >> 1)), packed 4 bits per pixel
    auto quad = [&](uint64_t m) {
      uint32_t r = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i)
        r |= (static_cast<uint32_t>(m >> (((qy + (i >> 1)) * 4 + qx + (i & 1)) * 4)) & 0xFu) << (4 * i);
      return r;
    };
    uint32_t const tq = quad(tz);
    if (!tq) continue;
    uint32_t const cq = quad(cv), uq = quad(uc);
    bool const fullq = full ? cq == qfull : (uq == qfull && cq == uq);
    uint32_t const ax = bx_abs + qx, ay = by_abs + qy;
    owner_append(P, L, rec, (ax >> 1) | ((ay >> 1) << 12) | (fullq ? 1u << 24 : 0u) | na, tq | (cq << 16));
  }
}

__global__ void __launch_bounds__(CV_THREADS) k_cover2(PassParams P) {
  extern __shared__ __align__(16) uint8_t smem[];
  TriCv* stage = reinterpret_cast<TriCv*>(smem);
  uint32_t* mask4 = reinterpret_cast<uint32_t*>(smem + CV_STAGE * sizeof(TriCv));  // [word][64 blocks]
  uint32_t* mask4f = mask4 + 64 * CV_WORDS;                                        // [word][64 blocks]
  uint32_t* mask16 = mask4f + 64 * CV_WORDS;                                       // [word][4 regions]
  uint32_t* ztile = mask16 + 4 * CV_WORDS;
  __shared__ uint32_t s_item;
  if (P.counters->overflow & (OVF_BIN | OVF_REC)) return;
  int const tid = threadIdx.x, h = tid & 1, ib = tid >> 1;  // item block 0..63: (ib & 7, ib >> 3)
  int const ibx = ib & 7, iby = ib >> 3;
  uint32_t const nitems = P.ntiles * 4;
  OwnerList L{NO_CHUNK, NO_CHUNK, 0};
  for (;;) {
    if (tid == 0) s_item = atomicAdd(&P.counters->tile_cursor, 1u);
    __syncthreads();
    uint32_t const item = s_item;
    __syncthreads();
    if (item >= nitems) break;
    uint32_t const tile = item >> 2, sub = item & 3;
    uint32_t const begin = P.tile_begin[tile], end = P.tile_begin[tile + 1];
    TargetParams const& T = P.targets[target_of_tile(P, tile)];
    uint32_t const ltile = tile - T.tile_base;
    int const tile_x0 = static_cast<int>(ltile % T.tiles_x) * TILE, tile_y0 = static_cast<int>(ltile / T.tiles_x) * TILE;
    int const bx0 = (sub & 1) * 8, by0 = (sub >> 1) * 8;  // first block of the quadrant, tile numbering
    int const x0 = tile_x0 + bx0 * 4, y0 = tile_y0 + by0 * 4;
    float const tx0f = static_cast<float>(tile_x0), ty0f = static_cast<float>(tile_y0);
    float const trr = T.target_w, trb = T.target_h;
    uint32_t const S = T.samples;
    int const bx = bx0 + ibx, by = by0 + iby;        // this thread's block, tile numbering
    int const bx_abs = tile_x0 + bx * 4, by_abs = tile_y0 + by * 4;
    int const own16 = (iby >> 2) * 2 + (ibx >> 2);  // its 16x16 region within the quadrant
    L.first = L.cur = NO_CHUNK;
    L.count = 0;
    Half hf;
    hf.s0 = S > 1 ? h * (S >> 1) : 0;
    hf.ns = S > 1 ? (S >> 1) : 1;
    hf.r0 = S > 1 ? 0 : 2 * h;
    hf.nr = S > 1 ? 4 : 2;
    hf.inside = 0;
    for (int iy = 0; iy < 4; ++iy)
      for (int ix = 0; ix < 4; ++ix)
        if (static_cast<uint32_t>(bx_abs + ix) < T.width && static_cast<uint32_t>(by_abs + iy) < T.height)
          hf.inside |= 1u << (iy * 4 + ix);
    bool const stage_z = T.any_early_z && begin < end;
    bool const d24 = T.ds_fmt == SG_FMT_D24S8;
    uint32_t const qw = min(static_cast<uint32_t>(CV_PX), T.width - min(T.width, static_cast<uint32_t>(x0)));
    uint32_t const qh = min(static_cast<uint32_t>(CV_PX), T.height - min(T.height, static_cast<uint32_t>(y0)));
    uint32_t const zrow = CV_PX * S;
    if (stage_z) {
      for (uint32_t i = tid; i < qh * zrow; i += CV_THREADS) {
        uint32_t y = i / zrow, k = i % zrow;
        if (k >= qw * S) continue;
        uint32_t x = k / S, sm = k % S;
        ztile[i] = *reinterpret_cast<uint32_t const*>(ds_addr(T, x0 + x, y0 + y, sm));
      }
    }
    uint32_t* const zblk = ztile + (iby * 4 * zrow) + ibx * 4 * S;
    ZRange zr{-INFINITY, INFINITY, 0u, 0xFFFFFFu};
    if (stage_z) {
      __syncthreads();
      z_range(zblk, static_cast<int>(zrow), S, hf, d24, zr);
    }
    for (uint32_t bstart = begin; bstart < end; bstart += CV_STAGE) {
      uint32_t const nb = min(static_cast<uint32_t>(CV_STAGE), end - bstart);
      __syncthreads();
      for (int i = tid; i < (64 + 64 + 4) * CV_WORDS; i += CV_THREADS) mask4[i] = 0;
      __syncthreads();
      // stage the batch and classify each triangle against the quadrant's regions and blocks
      for (uint32_t i = tid; i < nb; i += CV_THREADS) {
        uint32_t const e = P.bin_entries[bstart + i];
        float4 const* R = P.recs + (e >> 1);
        DrawParams const& D = P.draws[rec_draw(R)];
        int const nreg = 1 + static_cast<int>(D.nattr);
        TriCv ts;
        ts.e0 = R[0];
        ts.e1 = R[1];
        ts.e2 = R[2];
        ts.bbox = R[3];
        float4 const p0 = R[5];
        ts.p0x = p0.x;
        ts.p0y = p0.y;
        ts.p0z = p0.z;
        ts.dzx = R[5 + nreg].z;
        ts.dzy = R[5 + 2 * nreg].z;
        ts.entry = e;
        ts.zcfg = D.zcfg;
        ts.nattr = D.nattr;
        stage[i] = ts;
        uint32_t const bit = 1u << (i & 31), word = i >> 5;
        if (e & 1u) {  // accepted for the whole tile by the binner
          for (int r = 0; r < 4; ++r) atomicOr(&mask16[word * 4 + r], bit);
          continue;
        }
        float const x_min = ts.bbox.x - tx0f, x_max = ts.bbox.y - tx0f, y_min = ts.bbox.z - ty0f,
                    y_max = ts.bbox.w - ty0f;
        float4 const ed[3] = {ts.e0, ts.e1, ts.e2};
        LevelParams l1, l2;
        level_params(ed, l1, l2);
        for (int iy = by0 >> 2; iy < (by0 >> 2) + 2; ++iy) {
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
              atomicOr(&mask16[word * 4 + r], bit);
              continue;
            }
            // partial: level 2 over the 4x4 children inside the bounding box
            float const r16xf = static_cast<float>(tile_x0 + m16x), r16yf = static_cast<float>(tile_y0 + m16y);
            for (int jy = 0; jy < 4; ++jy) {
              int const m4y = m16y + jy * 4;
              if (y_min >= static_cast<float>(m4y + 4) || y_max < static_cast<float>(m4y)) continue;
              if (static_cast<float>(tile_y0 + m4y) >= trb) continue;
              for (int jx = 0; jx < 4; ++jx) {
                int const m4x = m16x + jx * 4;
                if (x_min >= static_cast<float>(m4x + 4) || x_max < static_cast<float>(m4x)) continue;
                if (static_cast<float>(tile_x0 + m4x) >= trr) continue;
                int const c2 = child_class(ed, l2, r16xf, r16yf, jx, jy);
                if (c2 == 0) continue;
                int const bi = (iy * 4 + jy - by0) * 8 + (ix * 4 + jx - bx0);
                atomicOr(&mask4[word * 64 + bi], bit);
                if (c2 == 2) atomicOr(&mask4f[word * 64 + bi], bit);
              }
            }
          }
        }
      }
      __syncthreads();
      // every block, by its two threads, walks its triangles in primitive order
      for (int w = 0; w < CV_WORDS; ++w) {
        uint32_t const m16 = mask16[w * 4 + own16];
        uint32_t mine = mask4[w * 64 + ib] | m16;
        uint32_t const fulls = mask4f[w * 64 + ib] | m16;
        while (mine) {
          int const b = __ffs(mine) - 1;
          mine &= mine - 1;
          cv_pair(P, T, stage[(w << 5) + b], (fulls >> b) & 1u, bx_abs, by_abs, zblk, static_cast<int>(zrow), h,
                  hf, zr, L);
        }
      }
    }
    if (stage_z) {
      __syncthreads();
      for (uint32_t i = tid; i < qh * zrow; i += CV_THREADS) {
        uint32_t y = i / zrow, k = i % zrow;
        if (k >= qw * S) continue;
        uint32_t x = k / S, sm = k % S;
        *reinterpret_cast<uint32_t*>(ds_addr(T, x0 + x, y0 + y, sm)) = ztile[i];
      }
    }
    // close the block's list for the item
    if (h == 0) {
      if (L.cur != NO_CHUNK) {
        P.chunk_next[L.cur] = NO_CHUNK;
        P.chunk_count[L.cur] = L.count;
      }
      P.owner_first[static_cast<size_t>(tile) * RASTER_THREADS + by * 16 + bx] = L.first;
    }
  }
}

void launch_cover2(PassParams const& p, uint32_t max_samples, bool early_z, uint32_t grid, cudaStream_t s) {
  k_cover2<<<grid, CV_THREADS, cv_smem(max_samples, early_z), s>>>(p);
}

cudaError_t init_cover2() {
  return cudaFuncSetAttribute(k_cover2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(cv_smem(4, true)));
}

}  // namespace sg
