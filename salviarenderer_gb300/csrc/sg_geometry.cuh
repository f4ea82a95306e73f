// sg_geometry.cuh -- the geometry kernel of a pass: one thread per input
// primitive of every draw: index fetch, vertex shader, near/far clipping and
// culling, viewport transform and projection, triangle setup (or segment
// records for lines) into compact records in slot order.  A template over
// the user vertex shader a pass runs: sg_draw.cu instantiates it for none,
// a user vertex-shader module for its own class.
#pragma once

#include <type_traits>

#include "sg_draw.cuh"

namespace sg {

// ---------------------------------------------------------------------------
// vertex processing
template <int NA>
struct vtx {
  v4 r[1 + NA];
};

// Reads past the end of a buffer are undefined in the reference; here they
// read zeros and are counted in fetch_oob.
__device__ inline uint32_t fetch_index(PassParams const& P, DrawParams const& D, uint32_t id) {
  if (!D.index_base) return id + static_cast<uint32_t>(D.base_vertex);
  if (id >= D.index_count) {
    atomicAdd(&P.counters->fetch_oob, 1u);
    return static_cast<uint32_t>(D.base_vertex);
  }
  uint32_t v = D.index_stride == 2 ? reinterpret_cast<uint16_t const*>(D.index_base)[id]
                                   : reinterpret_cast<uint32_t const*>(D.index_base)[id];
  return v + static_cast<uint32_t>(D.base_vertex);
}

// stream_assembler::fetch_vertex / get_vec4 (stream_assembler.cpp:26-93)
__device__ inline v4 fetch_input(PassParams const& P, DrawParams const& D, int r, uint32_t index) {
  uint32_t slot = D.in_slot[r];
  uint64_t off = static_cast<uint64_t>(D.stream_stride[slot]) * index + D.in_off[r];
  uint32_t n = D.in_fmt[r] == SG_VFMT_R32_FLOAT ? 4 : D.in_fmt[r] == SG_VFMT_R32G32_FLOAT ? 8
             : D.in_fmt[r] == SG_VFMT_R32G32B32_FLOAT ? 12 : 16;
  if (off + n > D.stream_bytes[slot] || (off & 3)) {
    atomicAdd(&P.counters->fetch_oob, 1u);
    return mk4(0, 0, 0, 0);
  }
  float const* f = reinterpret_cast<float const*>(D.stream_base[slot] + off);
  float dw = D.in_dw[r];
  switch (D.in_fmt[r]) {
  case SG_VFMT_R32_FLOAT: return mk4(f[0], 0.0f, 0.0f, dw);
  case SG_VFMT_R32G32_FLOAT: return mk4(f[0], f[1], 0.0f, dw);
  case SG_VFMT_R32G32B32_FLOAT: return mk4(f[0], f[1], f[2], dw);
  default: return mk4(f[0], f[1], f[2], f[3]);
  }
}

// eflib::transform(out, v, m) (eflib/src/math.cpp:142-154): out[j] = dot_prod4(v, column j)
__device__ inline v4 transform(v4 v, float const* m) {
  float o[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) o[j] = v.x * m[j] + v.y * m[4 + j] + v.z * m[8 + j] + v.w * m[12 + j];
  return mk4(o[0], o[1], o[2], o[3]);
}

// A user vertex shader's body on one vertex (defined with the user shader
// kernels, salvia_gb300/device_shader.cuh): the input registers to the
// position and the NA varyings.
template <class UVS, int NA>
__device__ void user_vs(DrawParams const& D, v4 const* in, v4* out);

// cpp_vertex_shader::execute (shader.cpp:520-522) for a stock program, or
// UVS's body for a user program
template <int NA, class UVS = void>
__device__ void run_vs(PassParams const& P, DrawParams const& D, uint32_t index, vtx<NA>& out) {
  v4 in[SG_MAX_VS_INPUTS];
#pragma unroll
  for (int r = 0; r < SG_MAX_VS_INPUTS; ++r) in[r] = mk4(0, 0, 0, 0);
  for (int r = 0; r < static_cast<int>(D.num_inputs); ++r) in[r] = fetch_input(P, D, r, index);
  if constexpr (!std::is_void<UVS>::value) {
    if (D.vs_prog >= SG_USER_PROGRAM_BASE) {
      user_vs<UVS, NA>(D, in, out.r);
      return;
    }
  }
  switch (D.vs_prog) {
  case SG_VS_TRANSFORM:
    out.r[0] = transform(in[0], D.vs_k);
#pragma unroll
    for (int i = 0; i < NA; ++i) out.r[1 + i] = in[1 + i];
    break;
  case SG_VS_MORPH_DISPLACE: {
    v4 pp = in[0] + (in[1] - in[0]) * D.vs_k[16];
    v4 n = in[2];
    float h = sample_impl(D.vs_samp, in[3].x, in[3].y, 0.0f, nullptr).x;
    float hs = h * D.vs_k[17];
    pp.x = pp.x + n.x * hs;
    pp.y = pp.y + n.y * hs;
    pp.z = pp.z + n.z * hs;
    out.r[0] = transform(pp, D.vs_k);
    if constexpr (NA > 0) out.r[1] = in[3];
    if constexpr (NA > 1) out.r[2] = n;
#pragma unroll
    for (int i = 2; i < NA; ++i) out.r[1 + i] = mk4(0, 0, 0, 0);
    break;
  }
  default:
    out.r[0] = mk4(0, 0, 0, 1);
#pragma unroll
    for (int i = 0; i < NA; ++i) out.r[1 + i] = mk4(0, 0, 0, 0);
    break;
  }
}

// cull functions (raster_state.cpp:10-32)
__device__ inline bool cull(DrawParams const& D, float area) {
  if (D.cull_mode == SG_CULL_NONE) return false;
  bool cull_ccw = (D.cull_mode == SG_CULL_FRONT) ? (D.front_ccw != 0) : (D.front_ccw == 0);
  return cull_ccw ? (area <= 0) : (area >= 0);
}

// vs_output_op lerp_n (shader.cpp:170-180)
template <int NA>
__device__ inline void vtx_lerp(DrawParams const& D, vtx<NA>& out, vtx<NA> const& a, vtx<NA> const& b, float t) {
  out.r[0] = a.r[0] + (b.r[0] - a.r[0]) * t;
#pragma unroll
  for (int i = 0; i < NA; ++i) {
    out.r[1 + i] = a.r[1 + i];
    if (!(D.mods[i] & SG_AM_NOINTERPOLATION)) out.r[1 + i] = out.r[1 + i] + (b.r[1 + i] - a.r[1 + i]) * t;
  }
}

__device__ inline float clip_d(int plane, v4 q) {  // dot_prod4 with planes (0,0,1,0), (0,0,-1,1)
  return plane == 0 ? (((0.0f * q.x + 0.0f * q.y) + 1.0f * q.z) + 0.0f * q.w)
                    : (((0.0f * q.x + 0.0f * q.y) + -1.0f * q.z) + 1.0f * q.w);
}

// viewport_transform + project_n (shader.cpp:499-511, 117-134)
template <int NA>
__device__ inline void vp_project(DrawParams const& D, vtx<NA>& v) {
  v4 q = v.r[0];
  float invw = eq_eps(q.w, 0.0f) ? 1.0f : 1.0f / q.w;
  v4 pos = q * invw;
  float ox = (D.vp_x + D.vp_w) * 0.5f;
  float oy = (D.vp_y + D.vp_h) * 0.5f;
  v.r[0] = mk4((D.vp_w * 0.5f) * pos.x + ox, (D.vp_h * 0.5f) * -pos.y + oy,
               (D.vp_maxz - D.vp_minz) * pos.z + D.vp_minz, invw);
#pragma unroll
  for (int i = 0; i < NA; ++i)
    if (!(D.mods[i] & SG_AM_NOPERSPECTIVE)) v.r[1 + i] = v.r[1 + i] * invw;
}

// rasterizer::compute_triangle_info (rasterizer.cpp:864-945) + compute_derivative_n
// (shader.cpp:414-449) of a projected triangle, written straight into its
// record (no zero-area triangle gets one).  The vertices are picked by
// register selects rather than through pointers, so that they stay in
// registers.
template <int NA>
__device__ void emit_triangle(PassParams const& P, DrawParams const& D, uint32_t draw, uint32_t slot, vtx<NA> a,
                              vtx<NA> b, vtx<NA> c, uint32_t& ntri) {
  ++ntri;
  vp_project(D, a);
  vp_project(D, b);
  vp_project(D, c);
  constexpr uint32_t STRIDE = rec_stride_for(NA);
  constexpr int R = 1 + NA;
  // v0: the vertex nearest the origin by |x| + |y| in double (rasterizer.cpp:880-899)
  double dist[3];
  dist[0] = fabs(static_cast<double>(a.r[0].x)) + fabs(static_cast<double>(a.r[0].y));
  dist[1] = fabs(static_cast<double>(b.r[0].x)) + fabs(static_cast<double>(b.r[0].y));
  dist[2] = fabs(static_cast<double>(c.r[0].x)) + fabs(static_cast<double>(c.r[0].y));
  int r0;
  if (dist[0] < dist[1])
    r0 = dist[0] < dist[2] ? 0 : 2;
  else
    r0 = dist[1] < dist[2] ? 1 : 2;
  int const r1 = (r0 + 1) % 3, r2 = (r1 + 1) % 3;
  auto pick = [&](int r, int i) -> v4 { return r == 0 ? a.r[i] : (r == 1 ? b.r[i] : c.r[i]); };
  v4 const p0 = pick(r0, 0), p1 = pick(r1, 0), p2 = pick(r2, 0);
  v4 const e01p = p1 - p0, e02p = p2 - p0;
  float const area = e02p.x * e01p.y - e02p.y * e01p.x;
  if (eq_eps(area, 0.0f)) {
    P.slot_rec[slot] = NO_REC;
    return;
  }
  uint32_t idx = atomicAdd(&P.counters->rec_units, STRIDE);
  if (idx > P.rec_capacity - STRIDE || P.rec_capacity < STRIDE) {
    atomicOr(&P.counters->overflow, OVF_REC);
    P.slot_rec[slot] = NO_REC;
    return;
  }
  float4* const rec = P.recs + idx;
  float const inv_area = 1.0f / area;
  v4 const pa = a.r[0], pb = b.r[0], pc = c.r[0];
  // edge factors, with v0's projected x, y, z beside them (what coverage and
  // early-Z read, in the first five slots)
  v4 const vp[3] = {pa, pb, pc};
  float const v0w[3] = {p0.x, p0.y, p0.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    v4 const sv = vp[i], ev = vp[(i + 1) % 3];
    rec[i] = make_float4(sv.y - ev.y, ev.x - sv.x, ev.x * sv.y - ev.y * sv.x, v0w[i]);
  }
  rec[3] = make_float4(smin(smin(pa.x, pb.x), pc.x), smax(smax(pa.x, pb.x), pc.x), smin(smin(pa.y, pb.y), pc.y),
                       smax(smax(pa.y, pb.y), pc.y));
  float const e01x = e01p.x, e01y = e01p.y, e02x = e02p.x, e02y = e02p.y;
  float dzx = 0.0f, dzy = 0.0f;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    v4 const q0 = pick(r0, i);
    v4 const e01 = pick(r1, i) - q0, e02 = pick(r2, i) - q0;
    float xd[4], yd[4];
    float const* p01 = &e01.x;
    float const* p02 = &e02.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      xd[k] = (p02[k] * e01y - p01[k] * e02y) * inv_area;
      yd[k] = (p01[k] * e02x - p02[k] * e01x) * inv_area;
    }
    rec[5 + i] = make_float4(q0.x, q0.y, q0.z, q0.w);
    rec[5 + R + i] = make_float4(xd[0], xd[1], xd[2], xd[3]);
    rec[5 + 2 * R + i] = make_float4(yd[0], yd[1], yd[2], yd[3]);
    if (i == 0) {
      dzx = xd[2];
      dzy = yd[2];
    }
  }
  rec[4] = make_float4(dzx, dzy, __uint_as_float(draw), __uint_as_float(rec_flags(area > 0.0f, D.shade_key, D.zcfg)));
  P.slot_rec[slot] = idx;
}

// A projected segment's record (the segment record layout) into `slot`.
template <int NA>
__device__ void emit_segment(PassParams const& P, DrawParams const& D, uint32_t draw, uint32_t slot, vtx<NA> const& a,
                             vtx<NA> const& b) {
  constexpr uint32_t STRIDE = rec_stride_for(NA);
  constexpr int R = 1 + NA;
  uint32_t idx = atomicAdd(&P.counters->rec_units, STRIDE);
  if (idx > P.rec_capacity - STRIDE || P.rec_capacity < STRIDE) {
    atomicOr(&P.counters->overflow, OVF_REC);
    idx = NO_REC;
  } else {
    float4* dst = P.recs + idx;
    float4 const never = make_float4(0.0f, 0.0f, -1.0f, 0.0f);
    dst[0] = never;
    dst[1] = never;
    dst[2] = never;
    // the box binning lists the segment under: its pixels' positions are
    // lerped, so widened past the rounding of the lerp (two units in the
    // last place of the largest coordinate, and two pixels), and bounded so
    // that the tile range stays in int
    v4 const pa = a.r[0], pb = b.r[0];
    float const mag = fmaxf(fmaxf(fabsf(pa.x), fabsf(pb.x)), fmaxf(fabsf(pa.y), fabsf(pb.y)));
    float const mg = 2.0f + mag * 0x1p-20f;
    auto bound = [](float v) { return fminf(fmaxf(v, -0x1p30f), 0x1p30f); };
    dst[3] = make_float4(bound(smin(pa.x, pb.x) - mg), bound(smax(pa.x, pb.x) + mg), bound(smin(pa.y, pb.y) - mg),
                         bound(smax(pa.y, pb.y) + mg));
    dst[4] = make_float4(0.0f, 0.0f, __uint_as_float(draw), __uint_as_float(rec_flags(true, D.shade_key, D.zcfg)));
#pragma unroll
    for (int i = 0; i < R; ++i) {
      dst[5 + i] = make_float4(a.r[i].x, a.r[i].y, a.r[i].z, a.r[i].w);
      dst[5 + R + i] = make_float4(b.r[i].x, b.r[i].y, b.r[i].z, b.r[i].w);
    }
  }
  P.slot_rec[slot] = idx;
}

// A triangle of the solid clipper drawn as its edges (a, b), (b, c), (c, a)
// into slots slot .. slot + 2.
template <int NA>
__device__ void emit_wire(PassParams const& P, DrawParams const& D, uint32_t draw, uint32_t slot, vtx<NA> a,
                          vtx<NA> b, vtx<NA> c, uint32_t& nseg) {
  nseg += 3;
  vp_project(D, a);
  vp_project(D, b);
  vp_project(D, c);
  emit_segment<NA>(P, D, draw, slot, a, b);
  emit_segment<NA>(P, D, draw, slot + 1, b, c);
  emit_segment<NA>(P, D, draw, slot + 2, c, a);
}

// The k-th output triangle of a primitive: a record, or (WIRE) three segments.
template <int NA, bool WIRE>
__device__ inline void emit_tri(PassParams const& P, DrawParams const& D, uint32_t draw, uint32_t slot0, int k,
                                vtx<NA> const& a, vtx<NA> const& b, vtx<NA> const& c, uint32_t& ntri) {
  if constexpr (WIRE)
    emit_wire<NA>(P, D, draw, slot0 + 3 * k, a, b, c, ntri);
  else
    emit_triangle<NA>(P, D, draw, slot0 + k, a, b, c, ntri);
}

// A line primitive: assembled (index_fetcher.cpp:53-60), shaded, cut at
// z >= 0 then z <= w (the outside end replaced by lerp(inside, outside,
// d_in / (d_in - d_out))), projected, one segment record.
template <int NA, class UVS = void>
__device__ void geometry_line(PassParams const& P, DrawParams const& D, uint32_t draw, uint32_t prim,
                              uint32_t& nseg) {
  uint32_t const i0 = D.strip ? prim : prim * 2;
  vtx<NA> v[2];
  run_vs<NA, UVS>(P, D, fetch_index(P, D, i0), v[0]);
  run_vs<NA, UVS>(P, D, fetch_index(P, D, i0 + 1), v[1]);
  uint32_t const slot = D.slot_base + prim;
#pragma unroll
  for (int pl = 0; pl < 2; ++pl) {
    float const da = clip_d(pl, v[0].r[0]), db = clip_d(pl, v[1].r[0]);
    if (da < 0.0f && db < 0.0f) {
      P.slot_rec[slot] = NO_REC;
      return;
    }
    vtx<NA> t;
    if (da >= 0.0f && db < 0.0f) {
      vtx_lerp(D, t, v[0], v[1], da / (da - db));
      v[1] = t;
    } else if (da < 0.0f && db >= 0.0f) {
      vtx_lerp(D, t, v[1], v[0], db / (db - da));
      v[0] = t;
    }
  }
  ++nseg;
  vp_project(D, v[0]);
  vp_project(D, v[1]);
  emit_segment<NA>(P, D, draw, slot, v[0], v[1]);
}

// clipper::clip_solid_triangle + clip_triangle_to_poly_general (clipper.cpp:43-228);
// WIRE: each output triangle as its three edges (9 slots per primitive)
template <int NA, bool WIRE = false, class UVS = void>
__device__ void geometry_prim(PassParams const& P, DrawParams const& D, uint32_t draw, uint32_t prim,
                              uint32_t& ntri) {
  uint32_t ids[3];
  if (D.strip) {
    ids[0] = prim;
    ids[1] = prim + 1;
    ids[2] = prim + 2;
    if (prim & 1) {
      uint32_t t = ids[0];
      ids[0] = ids[2];
      ids[2] = t;
    }
  } else {
    ids[0] = prim * 3;
    ids[1] = prim * 3 + 1;
    ids[2] = prim * 3 + 2;
  }
  vtx<NA> tv[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) run_vs<NA, UVS>(P, D, fetch_index(P, D, ids[i]), tv[i]);
  uint32_t slot0 = D.slot_base + prim * (WIRE ? 9u : 3u);
  if constexpr (WIRE) {
#pragma unroll
    for (int k = 0; k < 9; ++k) P.slot_rec[slot0 + k] = NO_REC;
  } else {
    P.slot_rec[slot0 + 1] = NO_REC;
    P.slot_rec[slot0 + 2] = NO_REC;
  }
  bool in_frustum = true;
#pragma unroll
  for (int pl = 0; pl < 2; ++pl)
#pragma unroll
    for (int v = 0; v < 3; ++v)
      if (clip_d(pl, tv[v].r[0]) < 0) in_frustum = false;
  if (in_frustum) {
    float pv[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      float iw = 1.0f / tv[i].r[0].w;
      pv[i][0] = tv[i].r[0].x * iw;
      pv[i][1] = tv[i].r[0].y * iw;
    }
    float area = (pv[2][0] - pv[0][0]) * (pv[1][1] - pv[0][1]) - (pv[2][1] - pv[0][1]) * (pv[1][0] - pv[0][0]);
    bool front = area > 0.0f;
    if (cull(D, front ? 1.0f : -1.0f)) {
      P.slot_rec[slot0] = NO_REC;
    } else if (front) {
      emit_tri<NA, WIRE>(P, D, draw, slot0, 0, tv[0], tv[1], tv[2], ntri);
    } else {
      emit_tri<NA, WIRE>(P, D, draw, slot0, 0, tv[0], tv[2], tv[1], ntri);
    }
    return;
  }
  // Sutherland-Hodgman against the near (z >= 0) and far (z <= w) planes.
  vtx<NA> pool[7];
  pool[0] = tv[0];
  pool[1] = tv[1];
  pool[2] = tv[2];
  int npool = 3;
  int poly[2][5];
  int n[2] = {3, 0};
  poly[0][0] = 0;
  poly[0][1] = 1;
  poly[0][2] = 2;
  int src = 0, dst = 1;
  bool is_front = false, culled = false;
  float d0 = 0.0f, d1 = 0.0f;
  for (int pl = 0; pl < 2 && !culled; ++pl) {
    n[dst] = 0;
    if (n[src] != 0) d0 = clip_d(pl, pool[poly[src][0]].r[0]);
    for (int i = 0, j = 1; i < n[src]; ++i, ++j) {
      j %= n[src];
      d1 = clip_d(pl, pool[poly[src][j]].r[0]);
      if (d0 >= 0.0f) {
        poly[dst][n[dst]++] = poly[src][i];
        if (d1 < 0.0f) {
          vtx_lerp(D, pool[npool], pool[poly[src][i]], pool[poly[src][j]], d0 / (d0 - d1));
          poly[dst][n[dst]++] = npool++;
        }
      } else if (d1 >= 0.0f) {
        vtx_lerp(D, pool[npool], pool[poly[src][j]], pool[poly[src][i]], d1 / (d1 - d0));
        poly[dst][n[dst]++] = npool++;
      }
      d0 = d1;
    }
    if (pl == 0 && n[dst] >= 3) {
      float pv[3][2];
      for (int i = 0; i < 3; ++i) {
        v4 q = pool[poly[dst][i]].r[0];
        float inv_abs_w = 1.0f / fabsf(q.w);
        pv[i][0] = q.x * inv_abs_w;
        pv[i][1] = q.y * inv_abs_w;
      }
      float area = (pv[2][0] - pv[0][0]) * (pv[1][1] - pv[0][1]) - (pv[2][1] - pv[0][1]) * (pv[1][0] - pv[0][0]);
      is_front = area > 0.0f;
      if (cull(D, area)) culled = true;
    }
    src ^= 1;
    dst ^= 1;
  }
  int nv = culled ? 0 : n[src];
  P.slot_rec[slot0] = NO_REC;
  for (int t = 1; t + 1 < nv; ++t) {
    int ia = poly[src][0], ib = poly[src][is_front ? t : t + 1], ic = poly[src][is_front ? t + 1 : t];
    emit_tri<NA, WIRE>(P, D, draw, slot0, t - 1, pool[ia], pool[ib], pool[ic], ntri);
  }
}

template <int NA, class UVS>
__device__ inline void geometry_any(PassParams const& P, DrawParams const& D, uint32_t draw, uint32_t prim,
                                    uint32_t& ntri) {
  if (D.line_mode == 1)
    geometry_line<NA, UVS>(P, D, draw, prim, ntri);
  else if (D.line_mode == 2)
    geometry_prim<NA, true, UVS>(P, D, draw, prim, ntri);
  else
    geometry_prim<NA, false, UVS>(P, D, draw, prim, ntri);
}

// The geometry of a pass, every draw; UVS: the user vertex shader the
// pass's user-program draws run (void: none).
template <class UVS>
__device__ __forceinline__ void geometry_pass(PassParams const& P) {
  if (pass_gated(P)) return;
  uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t ntri = 0, draw = 0xFFFFFFFFu, corners = 3;
  if (g < P.nprims) {
    draw = upper_index(P.draw_prim_base, P.ndraws, g);
    DrawParams const& D = P.draws[draw];
    uint32_t prim = g - D.prim_base;
    if (D.line_mode == 1) corners = 2;
    switch (D.nattr) {
    case 0: geometry_any<0, UVS>(P, D, draw, prim, ntri); break;
    case 1: geometry_any<1, UVS>(P, D, draw, prim, ntri); break;
    case 2: geometry_any<2, UVS>(P, D, draw, prim, ntri); break;
    case 3: geometry_any<3, UVS>(P, D, draw, prim, ntri); break;
    case 4: geometry_any<4, UVS>(P, D, draw, prim, ntri); break;
    default: geometry_any<5, UVS>(P, D, draw, prim, ntri); break;
    }
  }
  // per-draw counters, aggregated over the lanes of one draw: clipped
  // triangles (segments for lines), and vertex-shader runs (one per corner
  // of every primitive)
  uint32_t grp = __match_any_sync(0xFFFFFFFFu, draw);
  uint32_t sum = __reduce_add_sync(grp, ntri);
  uint32_t const leader = static_cast<uint32_t>(__ffs(grp) - 1);
  if (draw != 0xFFFFFFFFu && (threadIdx.x & 31) == leader) {
    if (sum) atomicAdd(&P.draw_stats[draw].cprimitives, static_cast<unsigned long long>(sum));
    atomicAdd(&P.draw_stats[draw].vs_invocations, static_cast<unsigned long long>(corners) * __popc(grp));
  }
}


}  // namespace sg
