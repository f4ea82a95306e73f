// sg_misc.cu -- clears and MSAA resolves (batched as jobs), mip generation.
#include <cuda_runtime.h>

#include <algorithm>

#include "sg_draw.cuh"
#include "sg_jobs.cuh"

namespace sg {

// surface::fill (surface.cpp:170-275): every texel gets the converted colour.
// Element sizes that divide 16 bytes are written as 16-byte stores of the
// replicated texel; 12-byte texels word by word.
__device__ void fill_job(SurfaceJob const& j, uint32_t part, uint32_t nparts) {
  size_t const stride = static_cast<size_t>(nparts) * blockDim.x;
  size_t const i0 = static_cast<size_t>(part) * blockDim.x + threadIdx.x;
  if (j.esz == 4 || j.esz == 8 || j.esz == 16) {
    uint4 v;
    uint32_t* pv = &v.x;
    for (int k = 0; k < 4; ++k) pv[k] = j.pattern[k % (j.esz / 4)];
    size_t const nvec = j.n * j.esz / 16, tail_bytes = j.n * j.esz - nvec * 16;
    uint4* d = reinterpret_cast<uint4*>(j.dst);
    for (size_t w = i0; w < nvec; w += stride) d[w] = v;
    uint32_t* t = reinterpret_cast<uint32_t*>(j.dst + nvec * 16);
    for (size_t w = i0; w < tail_bytes / 4; w += stride) t[w] = pv[w % 4];
  } else {
    uint32_t const words = j.esz / 4;
    uint32_t* d = reinterpret_cast<uint32_t*>(j.dst);
    size_t const nwords = j.n * words;
    for (size_t w = i0; w < nwords; w += stride) d[w] = j.pattern[w % words];
  }
}

// Depth-stencil clear of one flag (framebuffer::clear_depth_stencil,
// framebuffer.cpp:616-644) or of D24S8 (extension).
__device__ void clear_ds_job(SurfaceJob const& j, uint32_t part, uint32_t nparts) {
  size_t const stride = static_cast<size_t>(nparts) * blockDim.x;
  for (size_t i = static_cast<size_t>(part) * blockDim.x + threadIdx.x; i < j.n; i += stride) {
    if (j.fmt == SG_FMT_RG32F) {
      uint32_t* w = reinterpret_cast<uint32_t*>(j.dst) + 2 * i;
      if (j.flags & SG_CLEAR_DEPTH) w[0] = __float_as_uint(j.depth);
      if (j.flags & SG_CLEAR_STENCIL) w[1] = j.stencil;
    } else if (j.fmt == SG_FMT_D32F) {
      if (j.flags & SG_CLEAR_DEPTH) reinterpret_cast<float*>(j.dst)[i] = j.depth;
    } else {
      uint32_t* w = reinterpret_cast<uint32_t*>(j.dst) + i;
      uint32_t v = *w;
      if (j.flags & SG_CLEAR_DEPTH) {
        float c = fminf(fmaxf(j.depth, 0.0f), 1.0f) * 16777215.0f;
        v = (v & 0xFF000000u) | __float2uint_rn(c);
      }
      if (j.flags & SG_CLEAR_STENCIL) v = (v & 0x00FFFFFFu) | ((j.stencil & 0xFFu) << 24);
      *w = v;
    }
  }
}

// surface::resolve (surface.cpp:123-140): sum of samples in rgba32f, times
// 1/S (eflib's operator/= multiplies by the reciprocal).  Four-sample RGBA8
// reads one 16-byte vector per pixel.
__device__ void resolve_job(SurfaceJob const& j, uint32_t part, uint32_t nparts) {
  size_t const stride = static_cast<size_t>(nparts) * blockDim.x;
  uint32_t const samples = j.samples;
  float const inv = 1.0f / static_cast<float>(samples);
  for (size_t i = static_cast<size_t>(part) * blockDim.x + threadIdx.x; i < j.n; i += stride) {
    v4 c = mk4(0, 0, 0, 0);
    if (j.fmt == SG_FMT_RGBA8 && samples == 4) {
      uint4 s = reinterpret_cast<uint4 const*>(j.src)[i];
      uint32_t w[4] = {s.x, s.y, s.z, s.w};
#pragma unroll
      for (int k = 0; k < 4; ++k)
        c = c + unorm8_word_to_f(w[k], true);
    } else {
      for (uint32_t s = 0; s < samples; ++s) c = c + read_texel(j.fmt, j.src + (i * samples + s) * j.esz);
    }
    write_texel(j.dst_fmt, j.dst + i * fmt_bytes(j.dst_fmt), c * inv);
  }
}

// One launch runs a list of jobs: blockIdx.y selects the job, the x blocks
// stride over its elements.
__global__ void __launch_bounds__(256) k_jobs(JobList L) {
  pdl_wait();
  if (L.status) {  // a job of a pass: nothing after an overflow the host has not handled yet
    if (L.status[0] & OVF_FATAL) return;
    if (L.count_pass && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(&L.status[1], 1u);
  }
  SurfaceJob const& j = L.jobs[blockIdx.y];
  switch (j.kind) {
  case JOB_FILL: fill_job(j, blockIdx.x, gridDim.x); break;
  case JOB_CLEAR_DS: clear_ds_job(j, blockIdx.x, gridDim.x); break;
  default: resolve_job(j, blockIdx.x, gridDim.x); break;
  }
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

// Launches the jobs, JOBS_PER_LAUNCH per launch; returns the launch count.
// With `status`, the jobs belong to a pass (see JobList); `count_pass` makes
// the last launch count the pass as completed.
uint32_t launch_jobs(SurfaceJob const* jobs, uint32_t n, uint32_t num_sms, cudaStream_t s, unsigned int* status,
                     bool count_pass) {
  uint32_t launches = 0;
  for (uint32_t first = 0; first < n; first += JOBS_PER_LAUNCH) {
    JobList L;
    L.n = std::min<uint32_t>(JOBS_PER_LAUNCH, n - first);
    L.status = status;
    L.count_pass = count_pass && first + JOBS_PER_LAUNCH >= n ? 1u : 0u;
    size_t most = 0;
    for (uint32_t i = 0; i < L.n; ++i) {
      L.jobs[i] = jobs[first + i];
      most = std::max<size_t>(most, L.jobs[i].n * (L.jobs[i].kind == JOB_FILL ? L.jobs[i].esz / 4 : 1));
    }
    // enough x blocks for the largest job, at most 16 per SM
    uint32_t bx = static_cast<uint32_t>(std::min<size_t>((most + 1023) / 1024, static_cast<size_t>(num_sms) * 16));
    bx = std::max<uint32_t>(1, bx);
    launch_pdl(k_jobs, dim3(bx, L.n), 256, 0, s, L);
    ++launches;
  }
  return launches;
}

// copy_image_to_surface_impl (tex_io.cpp:27-53): each pixel of a decoded
// image (3 or 4 bytes, alpha 0 without an alpha channel) as color_rgba8,
// converted to the texture's format through color_rgba32f
// (pixel_format_convertor, color_convertors.cpp: to_rgba32f, then assign).
// Rows arrive in FreeImage's order, which is the surface's.  Grid-stride.
__global__ void __launch_bounds__(256) k_ingest(uint8_t const* src, uint32_t n, uint32_t channels, uint8_t* dst,
                                                uint32_t fmt) {
  uint32_t const esz = fmt_bytes(fmt);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint8_t const* p = src + static_cast<size_t>(i) * channels;
    uint32_t const a = channels == 4 ? p[3] : 0u;
    write_texel(fmt, dst + static_cast<size_t>(i) * esz, unorm8_to_f(p[0], p[1], p[2], a));
  }
}

// save_surface's conversion (tex_io.cpp:170-180): each texel of a
// 1-sample surface into BGRA8 or RGB32F through color_rgba32f.
__global__ void __launch_bounds__(256) k_export(uint8_t const* src, uint32_t n, uint32_t fmt, uint8_t* dst,
                                                uint32_t out_fmt) {
  uint32_t const esz = fmt_bytes(fmt), osz = fmt_bytes(out_fmt);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    write_texel(out_fmt, dst + static_cast<size_t>(i) * osz, read_texel(fmt, src + static_cast<size_t>(i) * esz));
}

void launch_ingest(uint8_t const* src, uint32_t n, uint32_t channels, uint8_t* dst, uint32_t fmt, uint32_t num_sms,
                   cudaStream_t s) {
  uint32_t const blocks = std::max(1u, std::min((n + 255) / 256, num_sms * 8));
  if (n) k_ingest<<<blocks, 256, 0, s>>>(src, n, channels, dst, fmt);
}

void launch_export(uint8_t const* src, uint32_t n, uint32_t fmt, uint8_t* dst, uint32_t out_fmt, uint32_t num_sms,
                   cudaStream_t s) {
  uint32_t const blocks = std::max(1u, std::min((n + 255) / 256, num_sms * 8));
  if (n) k_export<<<blocks, 256, 0, s>>>(src, n, fmt, dst, out_fmt);
}

void launch_mip(uint8_t const* src, uint32_t sw, uint32_t sh, uint8_t* dst, uint32_t dw, uint32_t dh,
                uint32_t samples, uint32_t fmt, uint32_t filter, cudaStream_t s) {
  uint32_t n = dw * dh * samples;
  if (n) k_mip<<<(n + 255) / 256, 256, 0, s>>>(src, sw, sh, dst, dw, dh, samples, fmt, filter);
}

}  // namespace sg
