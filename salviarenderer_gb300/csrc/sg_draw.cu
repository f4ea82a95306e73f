// sg_draw.cu -- geometry and binning kernels of a pass.
//
//   k_geometry   one thread per input primitive of the pass (all draws):
//                index fetch, vertex shader, near/far clipping and culling,
//                viewport transform and projection, triangle setup ->
//                compact triangle records in slot order.
//   k_bin<count/fill>   one warp per chunk of a target's triangle slots,
//                walking them in API order: the reference's per-tile trivial
//                reject/accept test, emitted into per-(tile, chunk) runs so
//                that every tile list comes out in API order without a sort.
//   k_scan_*     exclusive scan of the per-(tile, chunk) counts.
//   k_tile_ranges  per tile [begin, end) into the bin entries.
#include <cuda_runtime.h>

#include "sg_geometry.cuh"

namespace sg {

// the geometry kernel without user vertex shaders
__global__ void __launch_bounds__(128, 4) k_geometry(PassParams P) { geometry_pass<void>(P); }

// ---------------------------------------------------------------------------
// binning (rasterizer::threaded_dispatch_primitive, rasterizer.cpp:775-862)

// The per-tile test of a triangle spanning several tiles: trivial reject
// (the tile is dropped) and trivial accept (bit 0 of the entry).
struct TileTest {
  float ez[3], ex[3], ey[3], r2a[3];
  bool mx[3], my[3];
  __device__ void init(float4 const& e0, float4 const& e1, float4 const& e2) {
    float4 const e[3] = {e0, e1, e2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      ez[k] = e[k].z;
      ex[k] = e[k].x;
      ey[k] = e[k].y;
      mx[k] = e[k].x > 0;
      my[k] = e[k].y > 0;
      float stx = TILE * e[k].x, sty = TILE * e[k].y;
      r2a[k] = -fabsf(stx) - fabsf(sty);
    }
  }
  // bit 0: accepted; bit 1: not rejected
  __device__ int test(int x, int y) const {
    int rej = 0, acc = 1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float evv = ez[k] - (static_cast<float>(x + mx[k]) * TILE * ex[k] + static_cast<float>(y + my[k]) * TILE * ey[k]);
      rej |= (0 < evv);
      acc &= (r2a[k] >= evv);
    }
    return rej ? 0 : (2 | acc);
  }
};

// Tiles up to which one lane tests a triangle's tiles alone in the count pass.
constexpr int BIN_LANE_TILES = 8;

// k_bin<false> counts the entries of every (tile, chunk); k_bin<true> writes
// them, each (tile, chunk) run in slot order (API order).  A warp walks a
// chunk of a target's slots 32 at a time, every lane fetching its own slot's
// triangle.  Counting needs no order: each lane counts its own triangle's
// tiles (same-tile increments of a warp aggregated), and the warp tests the
// tiles of a triangle spanning more than BIN_LANE_TILES together.  Filling
// walks the 32 slots in order: a run of consecutive single-tile triangles is
// written in one step (lanes of one tile ranked by lane, one cursor update
// per tile), a triangle spanning several tiles by the whole warp.
template <bool FILL>
__global__ void __launch_bounds__(128) k_bin(PassParams P) {
  pdl_wait();
  uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= P.nchunks || pass_gated(P)) return;
  uint32_t const t = P.chunk_target[warp];
  TargetParams const& T = P.targets[t];
  uint32_t const c = warp - T.chunk_base, nch = T.nchunks;
  uint32_t const slot_end = T.slot_base + T.nslots;
  uint32_t begin = T.slot_base + c * T.chunk, end = min(begin + T.chunk, slot_end);
  int const tgx = T.tiles_x;
  uint32_t* cnt = P.bin_counts + T.count_base + c;
  uint32_t const lt_mask = (1u << lane) - 1u;
  for (uint32_t base = begin; base < end; base += 32) {
    uint32_t slot = base + lane;
    uint32_t rec = slot < end ? P.slot_rec[slot] : NO_REC;
    float4 e0 = make_float4(0, 0, 0, 0), e1 = e0, e2 = e0;
    int sx = 0, sy = 0, ex = 0, ey = 0;
    if (rec != NO_REC) {
      float4 const* R = P.recs + rec;
      e0 = R[0];
      e1 = R[1];
      e2 = R[2];
      float4 bb = R[3];
      DrawParams const& D = P.draws[rec_draw(R)];
      int const tx_n = D.tiles_x, ty_n = D.tiles_y;
      sx = min(fast_floori_f(smax(0.0f, bb.x) / TILE), tx_n);
      sy = min(fast_floori_f(smax(0.0f, bb.z) / TILE), ty_n);
      ex = min(fast_ceili_f(smax(0.0f, bb.y) / TILE) + 1, tx_n);
      ey = min(fast_ceili_f(smax(0.0f, bb.w) / TILE) + 1, ty_n);
      // finite inputs always land in [0, n]; the clamps only bound non-finite ones
      sx = max(sx, 0);
      sy = max(sy, 0);
      ex = max(ex, 0);
      ey = max(ey, 0);
    }
    bool const has = rec != NO_REC && sx < ex && sy < ey;
    // single-tile primitives are pushed without the tile tests (rasterizer.cpp:809-811)
    bool const single = has && sx + 1 == ex && sy + 1 == ey;
    int const w = ex - sx, nt = has ? w * (ey - sy) : 0;
    uint32_t const single_m = __ballot_sync(0xFFFFFFFFu, single);
    if (!FILL) {
      // singles: one aggregated increment per tile
      if (single) {
        uint32_t const tile = static_cast<uint32_t>(sy * tgx + sx);
        uint32_t const grp = __match_any_sync(single_m, tile);
        if ((grp & lt_mask) == 0) atomicAdd(cnt + static_cast<size_t>(tile) * nch, static_cast<uint32_t>(__popc(grp)));
      }
      // few tiles: each lane its own; many: the warp together
      bool const small = has && !single && nt <= BIN_LANE_TILES;
      if (small) {
        TileTest tt;
        tt.init(e0, e1, e2);
        for (int j = 0; j < nt; ++j) {
          int x = sx + j % w, y = sy + j / w;
          if (tt.test(x, y)) atomicAdd(cnt + static_cast<size_t>(y * tgx + x) * nch, 1u);
        }
      }
      uint32_t big = __ballot_sync(0xFFFFFFFFu, has && nt > BIN_LANE_TILES);
      while (big) {
        int i = __ffs(big) - 1;
        big &= big - 1;
        TileTest tt;
        tt.init(make_float4(__shfl_sync(0xFFFFFFFFu, e0.x, i), __shfl_sync(0xFFFFFFFFu, e0.y, i),
                            __shfl_sync(0xFFFFFFFFu, e0.z, i), 0.0f),
                make_float4(__shfl_sync(0xFFFFFFFFu, e1.x, i), __shfl_sync(0xFFFFFFFFu, e1.y, i),
                            __shfl_sync(0xFFFFFFFFu, e1.z, i), 0.0f),
                make_float4(__shfl_sync(0xFFFFFFFFu, e2.x, i), __shfl_sync(0xFFFFFFFFu, e2.y, i),
                            __shfl_sync(0xFFFFFFFFu, e2.z, i), 0.0f));
        int const tsx = __shfl_sync(0xFFFFFFFFu, sx, i), tsy = __shfl_sync(0xFFFFFFFFu, sy, i);
        int const tw = __shfl_sync(0xFFFFFFFFu, w, i), tn = __shfl_sync(0xFFFFFFFFu, nt, i);
        for (int j = lane; j < tn; j += 32) {
          int x = tsx + j % tw, y = tsy + j / tw;
          if (tt.test(x, y)) atomicAdd(cnt + static_cast<size_t>(y * tgx + x) * nch, 1u);
        }
      }
      continue;
    }
    // fill, in slot order
    uint32_t pending = __ballot_sync(0xFFFFFFFFu, has);
    uint32_t const multi_m = pending & ~single_m;
    while (pending) {
      uint32_t const next_multi = multi_m & pending;
      int const m = next_multi ? __ffs(next_multi) - 1 : 32;
      uint32_t const run = pending & single_m & (m == 32 ? 0xFFFFFFFFu : ((1u << m) - 1u));
      if (run) {
        if ((run >> lane) & 1u) {
          uint32_t const tile = static_cast<uint32_t>(sy * tgx + sx);
          uint32_t const grp = __match_any_sync(run, tile);
          int const leader = __ffs(grp) - 1;
          uint32_t* cc = cnt + static_cast<size_t>(tile) * nch;
          uint32_t pos = 0;
          if (lane == leader) {
            pos = *cc;
            *cc = pos + static_cast<uint32_t>(__popc(grp));
          }
          pos = __shfl_sync(grp, pos, leader) + static_cast<uint32_t>(__popc(grp & lt_mask));
          if (pos < P.bin_capacity) P.bin_entries[pos] = rec << 1;
        }
        pending &= ~run;
        __syncwarp();
      }
      if (m < 32) {
        pending &= ~(1u << m);
        uint32_t const r = __shfl_sync(0xFFFFFFFFu, rec, m);
        TileTest tt;
        tt.init(make_float4(__shfl_sync(0xFFFFFFFFu, e0.x, m), __shfl_sync(0xFFFFFFFFu, e0.y, m),
                            __shfl_sync(0xFFFFFFFFu, e0.z, m), 0.0f),
                make_float4(__shfl_sync(0xFFFFFFFFu, e1.x, m), __shfl_sync(0xFFFFFFFFu, e1.y, m),
                            __shfl_sync(0xFFFFFFFFu, e1.z, m), 0.0f),
                make_float4(__shfl_sync(0xFFFFFFFFu, e2.x, m), __shfl_sync(0xFFFFFFFFu, e2.y, m),
                            __shfl_sync(0xFFFFFFFFu, e2.z, m), 0.0f));
        int const tsx = __shfl_sync(0xFFFFFFFFu, sx, m), tsy = __shfl_sync(0xFFFFFFFFu, sy, m);
        int const tw = __shfl_sync(0xFFFFFFFFu, w, m), tn = __shfl_sync(0xFFFFFFFFu, nt, m);
        for (int j = lane; j < tn; j += 32) {
          int x = tsx + j % tw, y = tsy + j / tw;
          int const res = tt.test(x, y);
          if (res) {
            // the chunk's cursor of this tile: only this warp touches it; each
            // tile appears once per triangle, and the __syncwarp below orders
            // one step's update before the next step's read
            uint32_t* cc = cnt + static_cast<size_t>(y * tgx + x) * nch;
            uint32_t pos = *cc;
            *cc = pos + 1;
            if (pos < P.bin_capacity) P.bin_entries[pos] = (r << 1) | static_cast<uint32_t>(res & 1);
          }
        }
        __syncwarp();
      }
    }
  }
}

// ---------------------------------------------------------------------------
// exclusive scan of n uint32 values in place; block sums in `sums`
constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;

__device__ inline uint32_t block_exclusive_scan(uint32_t v, uint32_t* smem, uint32_t& total) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t s = lane < static_cast<int>(blockDim.x >> 5) ? smem[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= o) s += y;
    }
    smem[lane] = s;
  }
  __syncthreads();
  uint32_t warp_off = wid > 0 ? smem[wid - 1] : 0;
  total = smem[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + x - v;
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_local(uint32_t* data, size_t n, uint32_t* sums) {
  pdl_wait();
  __shared__ uint32_t smem[32];
  size_t base = static_cast<size_t>(blockIdx.x) * SCAN_BLOCK * SCAN_ITEMS + threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    v[i] = base + i < n ? data[base + i] : 0;
    s += v[i];
  }
  uint32_t total;
  uint32_t off = block_exclusive_scan(s, smem, total);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) data[base + i] = off;
    off += v[i];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// single-block scan of the block sums
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_sums(uint32_t* sums, uint32_t nsums, PassCounters* ctr) {
  pdl_wait();
  __shared__ uint32_t smem[32];
  uint32_t carry = 0;
  for (uint32_t start = 0; start < nsums; start += SCAN_BLOCK * SCAN_ITEMS) {
    uint32_t base = start + threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      v[i] = base + i < nsums ? sums[base + i] : 0;
      s += v[i];
    }
    uint32_t total;
    uint32_t off = block_exclusive_scan(s, smem, total) + carry;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      if (base + i < nsums) sums[base + i] = off;
      off += v[i];
    }
    carry += total;
  }
  if (threadIdx.x == 0) ctr->bin_entries = carry;
}

__global__ void k_scan_add(uint32_t* data, size_t n, uint32_t const* sums) {
  pdl_wait();
  size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) data[i] += sums[i / (SCAN_BLOCK * SCAN_ITEMS)];
}

// tile ranges from the scanned counts, and the overflow check
__global__ void k_tile_ranges(PassParams P) {
  pdl_wait();
  if (pass_gated(P)) return;
  uint32_t tile = blockIdx.x * blockDim.x + threadIdx.x;
  if (tile < P.ntiles) {
    uint32_t t = upper_index(P.target_tile_base, P.ntargets, tile);
    TargetParams const& T = P.targets[t];
    P.tile_begin[tile] = P.bin_counts[T.count_base + static_cast<size_t>(tile - T.tile_base) * T.nchunks];
  }
  if (tile == 0) {
    P.tile_begin[P.ntiles] = P.counters->bin_entries;
    if (P.counters->bin_entries > P.bin_capacity) atomicOr(&P.counters->overflow, OVF_BIN);
  }
}

// Longest-first order of the tiles for the coverage and merge passes, whose
// dynamic schedulers then start the costly tiles first: tiles by descending
// log2 of their bin entries (the order inside a bucket is free -- no result
// depends on the order tiles are taken in).  counts[0..31] count the
// buckets (phase 0), counts[32..63] are the buckets' cursors (phase 1).
__global__ void k_tile_order(PassParams P, uint32_t* counts, uint32_t phase) {
  pdl_wait();
  uint32_t const tile = blockIdx.x * blockDim.x + threadIdx.x;
  if (tile >= P.ntiles || pass_gated(P)) return;
  uint32_t const entries = P.tile_begin[tile + 1] - P.tile_begin[tile];
  uint32_t const b = 31u - static_cast<uint32_t>(__clz(entries | 1u));
  if (phase == 0) {
    atomicAdd(&counts[b], 1u);
    return;
  }
  uint32_t base = 0;
  for (uint32_t k = b + 1; k < 32; ++k) base += counts[k];
  P.tile_order[base + atomicAdd(&counts[32 + b], 1u)] = tile;
}

// The pass's fragments grouped by shade key -- shade class, then pixel-shader
// program -- so each shading instance walks only its own class, and its
// warps run one program (order is free: every fragment's colour has its own
// slot).  Phase 0 counts the keys, phase 1 scatters the fragment indices;
// one atomic per warp and key.
__global__ void __launch_bounds__(256) k_frag_classes(PassParams P, uint32_t phase) {
  pdl_wait();
  __shared__ uint32_t base[128];
  if ((P.counters->overflow & OVF_FATAL) || pass_gated(P)) return;
  uint32_t const nfrag = min(P.counters->chunk_total, P.chunk_capacity) * FRAG_CHUNK;
  if (phase == 1) {  // exclusive scan of the 128 key sizes
    if (threadIdx.x < 32) {
      uint32_t const* c = P.class_counts + 4 * threadIdx.x;
      uint32_t const c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3];
      uint32_t incl = c0 + c1 + c2 + c3;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t const y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (static_cast<int>(threadIdx.x) >= o) incl += y;
      }
      uint32_t const excl = incl - (c0 + c1 + c2 + c3);
      base[4 * threadIdx.x] = excl;
      base[4 * threadIdx.x + 1] = excl + c0;
      base[4 * threadIdx.x + 2] = excl + c0 + c1;
      base[4 * threadIdx.x + 3] = excl + c0 + c1 + c2;
    }
    __syncthreads();
  }
  int const lane = threadIdx.x & 31;
  uint32_t const stride = gridDim.x * blockDim.x;
  uint32_t const rounds = (nfrag + stride - 1) / stride;
  for (uint32_t it = 0; it < rounds; ++it) {
    uint32_t const f = blockIdx.x * blockDim.x + threadIdx.x + it * stride;
    bool const live = f < nfrag && (f % FRAG_CHUNK) < P.chunk_count[f / FRAG_CHUNK];
    uint32_t const cls = live ? P.frag_pos[f] >> 25 : 128u;  // the shade key
    unsigned const same = __match_any_sync(0xFFFFFFFFu, cls);
    int const leader = __ffs(same) - 1;
    if (!live) continue;
    uint32_t first = 0;
    if (lane == leader)
      first = atomicAdd(&P.class_counts[(phase == 0 ? 0u : 128u) + cls], static_cast<unsigned>(__popc(same)));
    if (phase == 0) continue;
    first = __shfl_sync(same, first, leader);
    P.frag_list[base[cls] + first + __popc(same & ((1u << lane) - 1u))] = f;
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
void launch_geometry(PassParams const& P, cudaStream_t s) {
  uint32_t blocks = (P.nprims + 127) / 128;
  if (blocks) k_geometry<<<blocks, 128, 0, s>>>(P);
}

void launch_bin(PassParams const& P, bool fill, cudaStream_t s) {
  uint32_t blocks = (P.nchunks * 32 + 127) / 128;
  if (!blocks) return;
  if (fill)
    launch_pdl(k_bin<true>, blocks, 128, 0, s, P);
  else
    launch_pdl(k_bin<false>, blocks, 128, 0, s, P);
}

// exclusive scan of `n` counts in place; `sums` needs ceil(n / 4096) entries
void launch_scan(uint32_t* data, size_t n, uint32_t* sums, PassCounters* ctr, cudaStream_t s) {
  size_t nblocks = (n + SCAN_BLOCK * SCAN_ITEMS - 1) / (SCAN_BLOCK * SCAN_ITEMS);
  if (nblocks == 0) return;
  launch_pdl(k_scan_local, static_cast<uint32_t>(nblocks), SCAN_BLOCK, 0, s, data, n, sums);
  launch_pdl(k_scan_sums, 1, SCAN_BLOCK, 0, s, sums, static_cast<uint32_t>(nblocks), ctr);
  launch_pdl(k_scan_add, static_cast<uint32_t>((n + 255) / 256), 256, 0, s, data, n, sums);
}

void launch_tile_ranges(PassParams const& P, cudaStream_t s) {
  launch_pdl(k_tile_ranges, (P.ntiles + 255) / 256, 256, 0, s, P);
}
// P.frag_list / P.class_counts (zeroed here) in scratch.
// With `counted`, the coverage pass counted the keys into zeroed counters
// already (cover_counts_classes): only the scatter runs.
cudaError_t launch_frag_classes(PassParams const& P, uint32_t num_sms, bool counted, cudaStream_t s) {
  if (!counted) {
    cudaError_t e = cudaMemsetAsync(P.class_counts, 0, 256 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    k_frag_classes<<<num_sms * 4, 256, 0, s>>>(P, 0u);
  }
  launch_pdl(k_frag_classes, num_sms * 4, 256, 0, s, P, 1u);
  return cudaGetLastError();
}

// P.tile_order (ntiles) and `counts` (64 words, zeroed by the caller at the
// pass's start) in scratch.
cudaError_t launch_tile_order(PassParams const& P, uint32_t* counts, cudaStream_t s) {
  uint32_t const blocks = (P.ntiles + 255) / 256;
  launch_pdl(k_tile_order, blocks, 256, 0, s, P, counts, 0u);
  launch_pdl(k_tile_order, blocks, 256, 0, s, P, counts, 1u);
  return cudaGetLastError();
}

cudaError_t upload_ewa_table_geometry(float const* tab, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_ewa, tab, 256 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

}  // namespace sg
