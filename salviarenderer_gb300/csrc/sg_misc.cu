// sg_misc.cu -- clears, MSAA resolve and mip generation.
#include <cuda_runtime.h>

#include <algorithm>

#include "sg_common.cuh"

namespace sg {

// surface::fill (surface.cpp:170-275): every texel gets the converted colour.
// The converted texel (1..16 bytes) is replicated with 4-byte stores when the
// element size allows, else byte by byte.
__global__ void k_fill(uint8_t* data, size_t nelem, uint32_t esz, uint4 pattern) {
  size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  uint32_t const* pat = &pattern.x;
  if (esz % 4 == 0) {
    uint32_t words = esz / 4;
    uint32_t* d = reinterpret_cast<uint32_t*>(data);
    size_t nwords = nelem * words;
    for (size_t w = i; w < nwords; w += stride) d[w] = pat[w % words];
  } else {
    uint8_t const* pb = reinterpret_cast<uint8_t const*>(pat);
    size_t nbytes = nelem * esz;
    for (size_t b = i; b < nbytes; b += stride) data[b] = pb[b % esz];
  }
}

// Depth-stencil clear of one flag (framebuffer::clear_depth_stencil,
// framebuffer.cpp:616-644) or of D24S8 (extension).
__global__ void k_clear_ds(uint8_t* data, size_t nelem, uint32_t fmt, uint32_t flags, float depth,
                           uint32_t stencil) {
  size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (; i < nelem; i += stride) {
    if (fmt == SG_FMT_RG32F) {
      uint32_t* w = reinterpret_cast<uint32_t*>(data) + 2 * i;
      if (flags & SG_CLEAR_DEPTH) w[0] = __float_as_uint(depth);
      if (flags & SG_CLEAR_STENCIL) w[1] = stencil;
    } else if (fmt == SG_FMT_D32F) {
      if (flags & SG_CLEAR_DEPTH) reinterpret_cast<float*>(data)[i] = depth;
    } else {
      uint32_t* w = reinterpret_cast<uint32_t*>(data) + i;
      uint32_t v = *w;
      if (flags & SG_CLEAR_DEPTH) {
        float c = fminf(fmaxf(depth, 0.0f), 1.0f) * 16777215.0f;
        v = (v & 0xFF000000u) | __float2uint_rn(c);
      }
      if (flags & SG_CLEAR_STENCIL) v = (v & 0x00FFFFFFu) | ((stencil & 0xFFu) << 24);
      *w = v;
    }
  }
}

// surface::resolve (surface.cpp:123-140): sum of samples in rgba32f, times 1/S.
__global__ void k_resolve(uint8_t const* src, uint8_t* dst, uint32_t npix, uint32_t samples, uint32_t fmt,
                          uint32_t dst_fmt) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  uint32_t esz = fmt_bytes(fmt);
  v4 c = mk4(0, 0, 0, 0);
  for (uint32_t s = 0; s < samples; ++s) c = c + read_texel(fmt, src + (static_cast<size_t>(i) * samples + s) * esz);
  float inv = 1.0f / static_cast<float>(samples);
  write_texel(dst_fmt, dst + static_cast<size_t>(i) * fmt_bytes(dst_fmt), c * inv);
}

// Four-sample RGBA8 resolve, one pixel per thread, 16-byte loads.
__global__ void k_resolve_rgba8x4(uint4 const* src, uint32_t* dst, uint32_t npix) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  uint4 s = src[i];
  v4 c = mk4(0, 0, 0, 0);
  uint32_t w[4] = {s.x, s.y, s.z, s.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) c = c + unorm8_to_f(w[k] & 0xFF, (w[k] >> 8) & 0xFF, (w[k] >> 16) & 0xFF, w[k] >> 24);
  c = c * 0.25f;
  dst[i] = f_to_unorm8(c.x) | (f_to_unorm8(c.y) << 8) | (f_to_unorm8(c.z) << 16) | (f_to_unorm8(c.w) << 24);
}

// surface::make_mip_surface (surface.cpp:53-92)
__global__ void k_mip(uint8_t const* src, uint32_t sw, uint32_t sh, uint8_t* dst, uint32_t dw, uint32_t dh,
                      uint32_t samples, uint32_t fmt, uint32_t filter) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dw * dh * samples) return;
  uint32_t s = i % samples, px = i / samples;
  uint32_t x = px % dw, y = px / dw;
  uint32_t esz = fmt_bytes(fmt);
  auto at = [&](uint32_t xx, uint32_t yy) {
    return src + ((static_cast<size_t>(yy) * sw + xx) * samples + s) * esz;
  };
  uint8_t* out = dst + (static_cast<size_t>(px) * samples + s) * esz;
  if (filter == SG_FILTER_POINT) {
    write_texel(fmt, out, read_texel(fmt, at(x * 2, y * 2)));
    return;
  }
  uint32_t x1 = min(x * 2 + 1, sw - 1), y1 = min(y * 2 + 1, sh - 1);
  v4 c0 = read_texel(fmt, at(x * 2, y * 2)), c1 = read_texel(fmt, at(x1, y * 2)),
     c2 = read_texel(fmt, at(x * 2, y1)), c3 = read_texel(fmt, at(x1, y1));
  write_texel(fmt, out, (((c0 + c1) + c2) + c3) * 0.25f);
}

void launch_fill(uint8_t* data, size_t nelem, uint32_t esz, uint4 pattern, cudaStream_t s) {
  size_t work = nelem * (esz % 4 == 0 ? esz / 4 : esz);
  uint32_t blocks = static_cast<uint32_t>(std::min<size_t>((work + 255) / 256, 152 * 16));
  if (blocks) k_fill<<<blocks, 256, 0, s>>>(data, nelem, esz, pattern);
}
void launch_clear_ds(uint8_t* data, size_t nelem, uint32_t fmt, uint32_t flags, float depth, uint32_t stencil,
                     cudaStream_t s) {
  uint32_t blocks = static_cast<uint32_t>(std::min<size_t>((nelem + 255) / 256, 152 * 16));
  if (blocks) k_clear_ds<<<blocks, 256, 0, s>>>(data, nelem, fmt, flags, depth, stencil);
}
void launch_resolve(uint8_t const* src, uint8_t* dst, uint32_t npix, uint32_t samples, uint32_t fmt,
                    uint32_t dst_fmt, cudaStream_t s) {
  if (!npix) return;
  if (fmt == SG_FMT_RGBA8 && dst_fmt == SG_FMT_RGBA8 && samples == 4)
    k_resolve_rgba8x4<<<(npix + 255) / 256, 256, 0, s>>>(reinterpret_cast<uint4 const*>(src),
                                                          reinterpret_cast<uint32_t*>(dst), npix);
  else
    k_resolve<<<(npix + 255) / 256, 256, 0, s>>>(src, dst, npix, samples, fmt, dst_fmt);
}
void launch_mip(uint8_t const* src, uint32_t sw, uint32_t sh, uint8_t* dst, uint32_t dw, uint32_t dh,
                uint32_t samples, uint32_t fmt, uint32_t filter, cudaStream_t s) {
  uint32_t n = dw * dh * samples;
  if (n) k_mip<<<(n + 255) / 256, 256, 0, s>>>(src, sw, sh, dst, dw, dh, samples, fmt, filter);
}

}  // namespace sg
