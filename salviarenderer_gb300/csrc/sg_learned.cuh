// sg_learned.cuh -- the learned anisotropic filter: a 24 -> 64 -> 64 -> 5
// MLP (GELU, BF16 weights and activations, FP32 accumulate) that predicts
// the sampler's anisotropic result (RGBA, as a correction of the mean of
// four bilinear taps along the major axis) and a confidence from the
// derivatives, the mip level and those taps.
#pragma once

#include <cstdint>

#include "sg_common.cuh"

namespace sg {

constexpr int AF_F = 24;     // input features
constexpr int AF_K1 = 32;    // features padded to a multiple of 16
constexpr int AF_H = 64;     // hidden width
constexpr int AF_O = 5;      // RGBA + confidence
constexpr int AF_N3 = 16;    // outputs padded to a multiple of 16
constexpr int AF_TILE = 128; // samples per tensor-core tile
// fp32 master parameters, in this order: W1 [64 x 24], b1 [64], W2 [64 x 64],
// b2 [64], W3 [5 x 64], b3 [5] (W[out][in])
constexpr int AF_OFF_W1 = 0, AF_OFF_B1 = AF_OFF_W1 + AF_H * AF_F, AF_OFF_W2 = AF_OFF_B1 + AF_H,
              AF_OFF_B2 = AF_OFF_W2 + AF_H * AF_H, AF_OFF_W3 = AF_OFF_B2 + AF_H, AF_OFF_B3 = AF_OFF_W3 + AF_O * AF_H,
              AF_PARAMS = AF_OFF_B3 + AF_O;

// BF16 operand images of the weights, already in the tensor cores' K-major
// core-matrix layout (sg_tc.cuh): W1 [64 x 32], W2 [64 x 64], W3 [16 x 64],
// and for the backward pass W3^T [64 x 16], W2^T [64 x 64].
constexpr int AF_IMG_W1 = 0, AF_IMG_W2 = AF_IMG_W1 + AF_H * AF_K1 * 2, AF_IMG_W3 = AF_IMG_W2 + AF_H * AF_H * 2,
              AF_IMG_W3T = AF_IMG_W3 + AF_N3 * AF_H * 2, AF_IMG_W2T = AF_IMG_W3T + AF_H * AF_N3 * 2,
              AF_IMG_BYTES = AF_IMG_W2T + AF_H * AF_H * 2;

// The 24 input features of one anisotropic lookup (sampler::sample_2d_grad
// with ddx = (dxu, dxv), ddy = (dyu, dyv)); `af` receives the reference's
// anisotropy measures (calc_anisotropic_info, sampler.cpp:875-958).
//   0-3   texel-space derivatives divided by the longer one's length
//   4     mip level of the probes / 8
//   5     log2 of the longer derivative's length / 8
//   6     probe count / 16
//   7     log2 of the anisotropy ratio (long / minor) / 4
//   8-23  RGBA of four bilinear taps at the probes' level, along the major
//         axis at -3/8, -1/8, 1/8, 3/8 of the probe span, filtered by the
//         texture units where the format allows (dev_sampler::af_tex)
// With the anisotropy measures `af` already computed (calc_af, bias 0).
__device__ inline void af_features_from(dev_sampler const& s, float u, float v, float dxu, float dxv, float dyu,
                                        float dyv, af_info const& af, float* f) {
  float const fw = static_cast<float>(s.width), fh = static_cast<float>(s.height);
  float const tx0 = dxu * fw, tx1 = dxv * fh, ty0 = dyu * fw, ty1 = dyv * fh;
  float const lx = sqrtf(tx0 * tx0 + tx1 * tx1), ly = sqrtf(ty0 * ty0 + ty1 * ty1);
  float const lmax = fmaxf(fmaxf(lx, ly), 1e-12f);
  float const lmin = fmaxf(fminf(lx, ly), 1e-12f);
  float const inv = 1.0f / lmax;
  f[0] = tx0 * inv;
  f[1] = tx1 * inv;
  f[2] = ty0 * inv;
  f[3] = ty1 * inv;
  f[4] = af.lod * 0.125f;
  f[5] = log2f(fmaxf(lmax, 1.0f)) * 0.125f;
  f[6] = af.probe_count * 0.0625f;
  f[7] = log2f(fmaxf(lmax / lmin, 1.0f)) * 0.25f;
  int const lo = fast_roundi_f(af.lod);
  int const min_lod = s.nlevels - 1;
  int const lvl = lo < 0 ? 0 : (lo > min_lod ? min_lod : lo);
  float const span = fmaxf(af.probe_count - 1.0f, 0.0f);
  unsigned long long const obj = s.af_tex[lvl];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float const t = (static_cast<float>(k) - 1.5f) * 0.25f * span;
    float const tu = u + af.du * t, tv = v + af.dv * t;
    float4 c;
    if (obj) {  // the texture units' bilinear filter (features need not match the sampler bit for bit)
      c = tex2D<float4>(obj, tu, tv);
      if (s.fmt == SG_FMT_BGRA8) c = make_float4(c.z, c.y, c.x, c.w);
    } else {
      v4 const p = sample_surface(s, lvl, tu, tv, SG_FILTER_LINEAR);
      c = make_float4(p.x, p.y, p.z, p.w);
    }
    f[8 + 4 * k] = c.x;
    f[9 + 4 * k] = c.y;
    f[10 + 4 * k] = c.z;
    f[11 + 4 * k] = c.w;
  }
}
__device__ inline void af_features(dev_sampler const& s, float u, float v, float dxu, float dxv, float dyu, float dyv,
                                   float* f, af_info& af) {
  calc_af(s, dxu, dxv, dyu, dyv, 0.0f, af);
  af_features_from(s, u, v, dxu, dxv, dyu, dyv, af, f);
}

// The filter's prediction is this mean of the four taps plus the network's
// colour outputs (a residual): channel c of feature row f.
__host__ __device__ inline float af_skip(float const* f, int c) {
  return 0.25f * ((f[8 + c] + f[12 + c]) + (f[16 + c] + f[20 + c]));
}

struct AfModelDev {
  float* params;        // fp32 master parameters
  uint8_t* img;         // AF_IMG_BYTES of BF16 operand images
  float* adam_m;        // Adam moments
  float* adam_v;
  float* grads;         // gradient accumulators (fp32)
};

}  // namespace sg
