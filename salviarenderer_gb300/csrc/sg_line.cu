// sg_line.cu -- rasterization, shading and output merging of line segments
// (line topologies, and triangles drawn with SG_FILL_WIREFRAME).
//
// The reference declares lines but stops at ef_unimplemented; its
// rasterize_line (rasterizer.cpp:60-213) holds the intended DDA, which
// include/salvia_gb300.h turns into a definition: along the major axis, the
// pixels [floori(floor(start + 0.5)), floori(end - 0.5)) clamped to the
// draw's viewport within the render area; each takes the endpoints'
// registers lerped at its centre, its minor coordinate floored from the
// lerped position; one pixel-shader run per pixel with ddx / ddy from the
// line's derivative registers; sample 0 through render_sample with the
// depth and stencil tests after shading.
//
// A line pass bins its segments into the 64x64 tiles of their bounding
// boxes (the segment records carry edge factors no tile test rejects), so
// every tile's list is in API order.  k_lines runs a CTA per tile at a
// time: the tile's segments one after another, the threads of the CTA on
// the segment's pixels inside the tile (a DDA gives each major coordinate
// one pixel, so they are distinct), shading and merging them in place.  A
// pixel belongs to one tile, so no two CTAs touch it, and the barrier
// between segments keeps API order.
#include "sg_raster.cuh"

namespace sg {

constexpr int LINE_THREADS = 64;  // a tile's extent along the major axis

// The pixel `t` of the segment's run inside the tile at (tx0, ty0): its
// DDA step, pixel shader and output merger.  Returns whether a pixel was
// shaded (for the draw's counters).
template <int NA>
__device__ bool line_pixel(TargetParams const& T, DrawParams const& D, float4 const* R, int tx0, int ty0, int t) {
  constexpr int RN = 1 + NA;
  v4 a[RN], b[RN], diff[RN];
#pragma unroll
  for (int k = 0; k < RN; ++k) {
    float4 const fa = R[5 + k], fb = R[5 + RN + k];
    a[k] = mk4(fa.x, fa.y, fa.z, fa.w);
    b[k] = mk4(fb.x, fb.y, fb.z, fb.w);
    diff[k] = b[k] - a[k];
  }
  v4 const dir = diff[0];
  // the draw's viewport within the render area
  int const left = fast_floori_f(smax(0.0f, D.vp_x)), top = fast_floori_f(smax(0.0f, D.vp_y));
  float const vr = D.vp_x + D.vp_w, vb = D.vp_y + D.vp_h;
  int const right = fast_floori_f(T.target_w < vr ? T.target_w : vr);
  int const bottom = fast_floori_f(T.target_h < vb ? T.target_h : vb);
  if (right <= left || bottom <= top) return false;
  bool const xmaj = fabsf(dir.x) > fabsf(dir.y);
  float diff_dir = xmaj ? dir.x : dir.y;
  bool const swap = diff_dir < 0.0f;
  if (swap) diff_dir = -diff_dir;
  v4 const* start = swap ? b : a;
  v4 const* end = swap ? a : b;
  float const s_major = xmaj ? start[0].x : start[0].y, e_major = xmaj ? end[0].x : end[0].y;
  int const lo = xmaj ? left : top, hi = xmaj ? right : bottom;
  int const mlo = xmaj ? top : left, mhi = xmaj ? bottom : right;
  int sx = fast_floori_f(fast_floor(s_major + 0.5f));
  int ex = fast_floori_f(e_major - 0.5f);
  sx = min(max(sx, lo), hi);  // (rasterize_line clamps the start to hi - 1: see the header)
  ex = min(max(ex, lo), hi);
  // this tile's part of the run
  int const t0 = xmaj ? tx0 : ty0, m0 = xmaj ? ty0 : tx0;
  int const i = max(sx, t0) + t;
  if (i >= min(ex, t0 + TILE)) return false;
  float const step = static_cast<float>(i) + 0.5f - s_major;
  float const tt = step / diff_dir;
  v4 px[RN];
  px[0] = start[0] + (end[0] - start[0]) * tt;  // lerp_n (shader.cpp:171-180)
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    px[1 + k] = start[1 + k];
    if (!(D.mods[k] & SG_AM_NOINTERPOLATION)) px[1 + k] = px[1 + k] + (end[1 + k] - start[1 + k]) * tt;
  }
  float const m = xmaj ? px[0].y : px[0].x;
  if (m >= static_cast<float>(mhi) || m < static_cast<float>(mlo)) return false;
  int const mi = fast_floori_f(m);
  if (mi >= mhi || mi < m0 || mi >= m0 + TILE) return false;  // the next tile along the minor axis has it
  uint32_t const x = static_cast<uint32_t>(xmaj ? i : mi), y = static_cast<uint32_t>(xmaj ? mi : i);
  // the line's derivative registers, diff * (diff.x / |diff.xy|^2) and
  // diff * (diff.y / |diff.xy|^2); the pixel and its neighbours one ddx /
  // one ddy along them, unprojected (unproject_n, shader.cpp:136-160)
  float const len_sqr = dir.x * dir.x + dir.y * dir.y;
  float const fx = dir.x / len_sqr, fy = dir.y / len_sqr;
  v4 nx[RN], ny[RN];
#pragma unroll
  for (int k = 0; k < RN; ++k) {
    bool const flat = k > 0 && (D.mods[k - 1] & SG_AM_NOINTERPOLATION);  // no derivative
    nx[k] = flat ? px[k] : px[k] + diff[k] * fx;
    ny[k] = flat ? px[k] : px[k] + diff[k] * fy;
  }
  float const iw = 1.0f / px[0].w, iwx = 1.0f / nx[0].w, iwy = 1.0f / ny[0].w;
  v4 attr[NA > 0 ? NA : 1], ax0 = mk4(0, 0, 0, 0), ay0 = mk4(0, 0, 0, 0);
  attr[0] = mk4(0, 0, 0, 0);
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    bool const np = (D.mods[k] & SG_AM_NOPERSPECTIVE) != 0;
    attr[k] = np ? px[1 + k] : px[1 + k] * iw;
    if (k == 0) {
      ax0 = np ? nx[1] : nx[1] * iwx;
      ay0 = np ? ny[1] : ny[1] * iwy;
    }
  }
  LineNb nb;
  nb.u0 = attr[0].x;
  nb.v0 = attr[0].y;
  nb.u1 = ax0.x;
  nb.v1 = ax0.y;
  nb.u2 = ay0.x;
  nb.v2 = ay0.y;
  nb.ws[0] = attr[0].w;
  nb.ws[1] = ax0.w;
  nb.ws[2] = ay0.w;
  bool keep = true;
  v4 const out = run_ps_nb<NA>(D, attr, nb, keep);
  if (keep) {
    // colours 1..: attributes 1.. of SG_PS_COLOR_MRT, else zero
    float4 more[SG_MAX_COLOR_TARGETS - 1];
#pragma unroll
    for (uint32_t k = 0; k + 1 < SG_MAX_COLOR_TARGETS; ++k) {
      v4 c = mk4(0, 0, 0, 0);
#pragma unroll
      for (int j = 1; j < NA; ++j)
        if (D.ps_prog == SG_PS_COLOR_MRT && static_cast<uint32_t>(j) == k + 1) c = attr[j];
      more[k] = make_float4(c.x, c.y, c.z, c.w);
    }
    render_sample<void>(T, D, x, y, 0, out, px[0].z, true, more);
  }
  return true;
}

__global__ void __launch_bounds__(LINE_THREADS) k_lines(PassParams P) {
  pdl_wait();
  if (pass_gated(P)) return;
  uint32_t const ovf = P.counters->overflow;  // final: geometry and binning are done
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (ovf) atomicOr(P.sticky, ovf);
    if (P.count_pass && !(ovf & OVF_FATAL)) atomicAdd(P.sticky + 1, 1u);
  }
  if (ovf & OVF_FATAL) return;
  int const t = threadIdx.x;
  for (uint32_t tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
    uint32_t const begin = P.tile_begin[tile], end = P.tile_begin[tile + 1];
    if (begin == end) continue;
    TargetParams const& T = P.targets[target_of_tile(P, tile)];
    uint32_t const ltile = tile - T.tile_base;
    int const tx0 = static_cast<int>(ltile % static_cast<uint32_t>(T.tiles_x)) * TILE;
    int const ty0 = static_cast<int>(ltile / static_cast<uint32_t>(T.tiles_x)) * TILE;
    for (uint32_t e = begin; e < end; ++e) {
      float4 const* R = P.recs + (P.bin_entries[e] >> 1);
      uint32_t const draw = rec_draw(R);
      DrawParams const& D = P.draws[draw];
      bool shaded;
      switch (D.nattr) {
      case 0: shaded = line_pixel<0>(T, D, R, tx0, ty0, t); break;
      case 1: shaded = line_pixel<1>(T, D, R, tx0, ty0, t); break;
      case 2: shaded = line_pixel<2>(T, D, R, tx0, ty0, t); break;
      case 3: shaded = line_pixel<3>(T, D, R, tx0, ty0, t); break;
      case 4: shaded = line_pixel<4>(T, D, R, tx0, ty0, t); break;
      default: shaded = line_pixel<5>(T, D, R, tx0, ty0, t); break;
      }
      // ps_invocations and backend_input_pixels: one per shaded pixel
      unsigned const n = __popc(__ballot_sync(0xFFFFFFFFu, shaded));
      if ((t & 31) == 0 && n) {
        atomicAdd(&P.draw_stats[draw].ps_invocations, static_cast<unsigned long long>(n));
        atomicAdd(&P.draw_stats[draw].backend_input_pixels, static_cast<unsigned long long>(n));
      }
      __syncthreads();  // the next segment sees this one's writes (API order)
    }
  }
}

void launch_lines(PassParams const& p, uint32_t grid, cudaStream_t s) {
  launch_pdl(k_lines, grid, LINE_THREADS, 0, s, p);
}

// The EWA table of this translation unit's sampler.
cudaError_t upload_ewa_table_line(float const* tab, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_ewa, tab, 256 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

}  // namespace sg
