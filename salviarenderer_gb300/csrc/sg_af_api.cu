// sg_af_api.cu -- host runtime of the learned anisotropic filter: model
// creation and parameters, tensor-core inference, training (sampling the
// plain anisotropic sampler on the device, forward and backward passes,
// Adam) and evaluation against the plain sampler.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "salvia_gb300.h"
#include "sg_learned.cuh"

namespace sg {
cudaStream_t device_stream(sg_device* d);
int32_t device_settle(sg_device* d);
int device_sms(sg_device* d);
void device_set_error(sg_device* d, char const* msg);
int32_t device_af_sampler(sg_device* d, uint32_t handle, dev_sampler& out);
uint32_t device_register_af(sg_device* d, AfModelDev const& m);
uint8_t* device_texture_data(sg_device* d, uint32_t tex);
void launch_af_pattern(uint8_t* dst, uint32_t size, uint64_t seed, uint32_t index, cudaStream_t s);
void device_unregister_af(sg_device* d, uint32_t id);
void launch_af_pack(AfModelDev const& M, cudaStream_t s);
cudaError_t launch_af_infer(AfModelDev const& M, uint16_t const* X, float4 const* skip, uint32_t n, float* out,
                            unsigned int* status, uint32_t num_sms, cudaStream_t s);
cudaError_t launch_af_train(AfModelDev const& M, uint16_t const* X, float4 const* Y, uint32_t n, float inv_batch,
                            float* loss_out, unsigned int* status, uint32_t num_sms, cudaStream_t s);
void launch_af_adam(AfModelDev const& M, float lr, uint32_t step, cudaStream_t s);
void launch_af_samples(dev_sampler const* samplers, uint32_t ntex, uint32_t n, uint32_t first, uint64_t seed,
                       uint16_t* X, float4* Y, float* features_f32, bool residual, cudaStream_t s);
}  // namespace sg

using namespace sg;

struct sg_af_model {
  AfModelDev m{};
  unsigned int* status = nullptr;  // device: bit 0 a tensor-core wait timed out
  uint32_t steps = 0;              // Adam steps taken
  uint32_t id = 0;                 // the id draws name it by
};

namespace {

int32_t fail(sg_device* d, cudaError_t e, char const* what) {
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  device_set_error(d, msg.c_str());
  return e == cudaErrorMemoryAllocation ? SG_OUT_OF_MEMORY : SG_CUDA_ERROR;
}
#define AF_CUDA(d, call)                             \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return fail(d, e_, #call); \
  } while (0)

// BF16 bits of a float, round to nearest even (host side).
uint16_t host_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return static_cast<uint16_t>((u >> 16) | ((u & 0xFFFFu) ? 0x40u : 0u));
  uint32_t const lsb = (u >> 16) & 1u;
  u += 0x7FFFu + lsb;
  return static_cast<uint16_t>(u >> 16);
}

// splitmix64 stream for the initial weights
uint64_t mix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
float uniform(uint64_t& s) { return static_cast<float>((mix(s) >> 40) * (1.0 / 16777216.0)); }

int32_t check_status(sg_device* d, sg_af_model* m) {
  unsigned int st = 0;
  AF_CUDA(d, cudaMemcpyAsync(&st, m->status, 4, cudaMemcpyDeviceToHost, device_stream(d)));
  AF_CUDA(d, cudaStreamSynchronize(device_stream(d)));
  if (st) {
    device_set_error(d, "a tensor-core wait timed out");
    AF_CUDA(d, cudaMemset(m->status, 0, 4));
    return SG_TIMEOUT;
  }
  return SG_OK;
}

// Feature rows as the tensor cores read them (BF16, padded to 32 columns)
// and the fp32 tap means the prediction adds.
void stage_rows(float const* features, uint32_t n, std::vector<uint16_t>& x, std::vector<float>& skip) {
  x.assign(static_cast<size_t>(n) * AF_K1, 0);
  skip.resize(static_cast<size_t>(n) * 4);
  for (size_t r = 0; r < n; ++r) {
    float const* f = features + r * AF_F;
    for (int k = 0; k < AF_F; ++k) x[r * AF_K1 + k] = host_bf16(f[k]);
    for (int c = 0; c < 4; ++c) skip[r * 4 + c] = af_skip(f, c);
  }
}

// A device allocation released with its scope (cudaFree waits for the
// device's work in flight, so an early return frees nothing still in use).
template <class T>
struct DevBuf {
  T* p = nullptr;
  cudaError_t alloc(size_t count) { return cudaMalloc(&p, count * sizeof(T)); }
  ~DevBuf() { cudaFree(p); }
};

struct DevSamplers {
  DevBuf<dev_sampler> buf;
  dev_sampler* p = nullptr;
};

// The device images of sampler handles (textures stay where they are).
int32_t upload_samplers(sg_device* d, uint32_t const* handles, uint32_t n, DevSamplers& out) {
  std::vector<dev_sampler> h(n);
  for (uint32_t i = 0; i < n; ++i) {
    if (!handles[i]) return SG_INVALID_PARAMETER;
    if (int32_t r = device_af_sampler(d, handles[i], h[i])) return r;
  }
  AF_CUDA(d, out.buf.alloc(n));
  AF_CUDA(d, cudaMemcpyAsync(out.buf.p, h.data(), n * sizeof(dev_sampler), cudaMemcpyHostToDevice, device_stream(d)));
  out.p = out.buf.p;
  return SG_OK;
}

}  // namespace

extern "C" {

int32_t sg_af_model_create(sg_device* d, uint64_t seed, sg_af_model** out) {
  if (!d || !out) return SG_INVALID_PARAMETER;
  *out = nullptr;
  auto* m = new sg_af_model();
  cudaStream_t s = device_stream(d);
  size_t const pbytes = AF_PARAMS * sizeof(float);
  cudaError_t e = cudaMalloc(&m->m.params, pbytes);
  if (e == cudaSuccess) e = cudaMalloc(&m->m.img, AF_IMG_BYTES);
  if (e == cudaSuccess) e = cudaMalloc(&m->m.adam_m, pbytes);
  if (e == cudaSuccess) e = cudaMalloc(&m->m.adam_v, pbytes);
  if (e == cudaSuccess) e = cudaMalloc(&m->m.grads, pbytes + 64);
  if (e == cudaSuccess) e = cudaMalloc(&m->status, 4);
  if (e != cudaSuccess) {
    sg_af_model_destroy(d, m);
    return fail(d, e, "sg_af_model_create");
  }
  // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases
  std::vector<float> p(AF_PARAMS, 0.0f);
  uint64_t st = seed;
  auto fill = [&](int off, int count, int fan_in) {
    float const a = 1.0f / std::sqrt(static_cast<float>(fan_in));
    for (int i = 0; i < count; ++i) p[off + i] = (2.0f * uniform(st) - 1.0f) * a;
  };
  fill(AF_OFF_W1, AF_H * AF_F, AF_F);
  fill(AF_OFF_W2, AF_H * AF_H, AF_H);
  fill(AF_OFF_W3, AF_O * AF_H, AF_H);
  e = cudaMemcpyAsync(m->m.params, p.data(), pbytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->m.adam_m, 0, pbytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->m.adam_v, 0, pbytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->status, 0, 4, s);
  if (e == cudaSuccess) {
    launch_af_pack(m->m, s);
    e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess) {
    sg_af_model_destroy(d, m);
    return fail(d, e, "sg_af_model_create");
  }
  m->id = device_register_af(d, m->m);
  *out = m;
  return SG_OK;
}

uint32_t sg_af_model_id(const sg_af_model* m) { return m ? m->id : 0u; }

void sg_af_model_destroy(sg_device* d, sg_af_model* m) {
  if (!m) return;
  if (d) device_settle(d);  // a replay of logged passes reads the model
  if (d && m->id) device_unregister_af(d, m->id);
  if (d) cudaStreamSynchronize(device_stream(d));
  cudaFree(m->m.params);
  cudaFree(m->m.img);
  cudaFree(m->m.adam_m);
  cudaFree(m->m.adam_v);
  cudaFree(m->m.grads);
  cudaFree(m->status);
  delete m;
}

int32_t sg_af_model_get_params(sg_device* d, sg_af_model* m, float* params) {
  if (!d || !m || !params) return SG_INVALID_PARAMETER;
  AF_CUDA(d, cudaMemcpyAsync(params, m->m.params, AF_PARAMS * sizeof(float), cudaMemcpyDeviceToHost,
                             device_stream(d)));
  AF_CUDA(d, cudaStreamSynchronize(device_stream(d)));
  return SG_OK;
}

int32_t sg_af_model_set_params(sg_device* d, sg_af_model* m, const float* params) {
  if (!d || !m || !params) return SG_INVALID_PARAMETER;
  if (int32_t r = device_settle(d)) return r;
  cudaStream_t s = device_stream(d);
  AF_CUDA(d, cudaMemcpyAsync(m->m.params, params, AF_PARAMS * sizeof(float), cudaMemcpyHostToDevice, s));
  launch_af_pack(m->m, s);
  AF_CUDA(d, cudaStreamSynchronize(s));
  return SG_OK;
}

int32_t sg_af_model_forward(sg_device* d, sg_af_model* m, const float* features, uint32_t n, float* out) {
  if (!d || !m || (!features && n) || (!out && n)) return SG_INVALID_PARAMETER;
  if (n == 0) return SG_OK;
  cudaStream_t s = device_stream(d);
  std::vector<uint16_t> x;
  std::vector<float> skip;
  stage_rows(features, n, x, skip);
  DevBuf<uint16_t> X;
  DevBuf<float> K, O;
  AF_CUDA(d, X.alloc(x.size()));
  AF_CUDA(d, K.alloc(skip.size()));
  AF_CUDA(d, O.alloc(static_cast<size_t>(n) * 8));
  AF_CUDA(d, cudaMemcpyAsync(X.p, x.data(), x.size() * 2, cudaMemcpyHostToDevice, s));
  AF_CUDA(d, cudaMemcpyAsync(K.p, skip.data(), skip.size() * 4, cudaMemcpyHostToDevice, s));
  AF_CUDA(d, launch_af_infer(m->m, X.p, reinterpret_cast<float4 const*>(K.p), n, O.p, m->status,
                             static_cast<uint32_t>(device_sms(d)), s));
  std::vector<float> o(static_cast<size_t>(n) * 8);
  AF_CUDA(d, cudaMemcpyAsync(o.data(), O.p, o.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
  AF_CUDA(d, cudaStreamSynchronize(s));
  for (size_t r = 0; r < n; ++r)
    for (int k = 0; k < AF_O; ++k) out[r * AF_O + k] = o[r * 8 + k];
  return check_status(d, m);
}

int32_t sg_af_sample(sg_device* d, const uint32_t* samplers, uint32_t nsamp, uint32_t n, uint64_t seed,
                     float* features, float* targets) {
  if (!d || !samplers || nsamp == 0 || (n && (!features || !targets))) return SG_INVALID_PARAMETER;
  if (n == 0) return SG_OK;
  cudaStream_t s = device_stream(d);
  DevSamplers ds;
  if (int32_t r = upload_samplers(d, samplers, nsamp, ds)) return r;
  DevBuf<uint16_t> X;
  DevBuf<float4> Y;
  DevBuf<float> F;
  AF_CUDA(d, X.alloc(static_cast<size_t>(n) * AF_K1));
  AF_CUDA(d, Y.alloc(n));
  AF_CUDA(d, F.alloc(static_cast<size_t>(n) * AF_F));
  launch_af_samples(ds.p, nsamp, n, 0, seed, X.p, Y.p, F.p, false, s);
  AF_CUDA(d, cudaGetLastError());
  AF_CUDA(d, cudaMemcpyAsync(features, F.p, static_cast<size_t>(n) * AF_F * 4, cudaMemcpyDeviceToHost, s));
  AF_CUDA(d, cudaMemcpyAsync(targets, Y.p, static_cast<size_t>(n) * 16, cudaMemcpyDeviceToHost, s));
  AF_CUDA(d, cudaStreamSynchronize(s));
  return SG_OK;
}

int32_t sg_af_model_gradients(sg_device* d, sg_af_model* m, const float* features, const float* targets,
                              uint32_t n, float* grads, float* loss) {
  if (!d || !m || !features || !targets || !grads || n == 0) return SG_INVALID_PARAMETER;
  cudaStream_t s = device_stream(d);
  std::vector<uint16_t> x;
  std::vector<float> skip;
  stage_rows(features, n, x, skip);
  for (size_t i = 0; i < skip.size(); ++i) skip[i] = targets[i] - skip[i];  // the network's residual target
  DevBuf<uint16_t> X;
  DevBuf<float4> Y;
  DevBuf<float> L;
  AF_CUDA(d, X.alloc(x.size()));
  AF_CUDA(d, Y.alloc(n));
  AF_CUDA(d, L.alloc(1));
  AF_CUDA(d, cudaMemcpyAsync(X.p, x.data(), x.size() * 2, cudaMemcpyHostToDevice, s));
  AF_CUDA(d, cudaMemcpyAsync(Y.p, skip.data(), static_cast<size_t>(n) * 16, cudaMemcpyHostToDevice, s));
  AF_CUDA(d, cudaMemsetAsync(L.p, 0, 4, s));
  AF_CUDA(d, cudaMemsetAsync(m->m.grads, 0, AF_PARAMS * sizeof(float), s));
  AF_CUDA(d, launch_af_train(m->m, X.p, Y.p, n, 1.0f / static_cast<float>(n), L.p, m->status,
                             static_cast<uint32_t>(device_sms(d)), s));
  AF_CUDA(d, cudaMemcpyAsync(grads, m->m.grads, AF_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, s));
  float l = 0.0f;
  AF_CUDA(d, cudaMemcpyAsync(&l, L.p, 4, cudaMemcpyDeviceToHost, s));
  AF_CUDA(d, cudaMemsetAsync(m->m.grads, 0, AF_PARAMS * sizeof(float), s));
  AF_CUDA(d, cudaStreamSynchronize(s));
  if (loss) *loss = l / static_cast<float>(n);
  return check_status(d, m);
}

int32_t sg_af_make_textures(sg_device* d, uint32_t count, uint32_t size, uint64_t seed, uint32_t* out) {
  if (!d || !out || count == 0 || size < 16 || size > 4096 || (size & (size - 1))) return SG_INVALID_PARAMETER;
  for (uint32_t i = 0; i < count; ++i) {
    uint32_t h = 0;
    if (int32_t r = sg_texture_create(d, size, size, 1, SG_FMT_RGBA8, &h)) return r;
    out[i] = h;
    launch_af_pattern(device_texture_data(d, h), size, seed, i, device_stream(d));
    AF_CUDA(d, cudaGetLastError());
    if (int32_t r = sg_texture_gen_mipmap(d, h, SG_FILTER_LINEAR)) return r;
  }
  return SG_OK;
}

int32_t sg_af_model_train(sg_device* d, sg_af_model* m, const sg_af_train_desc* t, sg_af_report* rep) {
  if (!d || !m || !t || !t->samplers || t->num_samplers == 0 || t->samples == 0 || t->batch == 0 ||
      t->epochs == 0 || !(t->lr > 0.0f))
    return SG_INVALID_PARAMETER;
  if (int32_t r = device_settle(d)) return r;
  cudaStream_t s = device_stream(d);
  DevSamplers ds;
  if (int32_t r = upload_samplers(d, t->samplers, t->num_samplers, ds)) return r;
  uint32_t const n = t->samples;
  DevBuf<uint16_t> X;
  DevBuf<float4> Y;
  DevBuf<float> L;
  AF_CUDA(d, X.alloc(static_cast<size_t>(n) * AF_K1));
  AF_CUDA(d, Y.alloc(n));
  uint32_t const steps_per_epoch = (n + t->batch - 1) / t->batch;
  uint32_t const steps = steps_per_epoch * t->epochs;
  AF_CUDA(d, L.alloc(steps));
  AF_CUDA(d, cudaMemsetAsync(L.p, 0, steps * sizeof(float), s));
  // the training set, drawn once on the device from the plain sampler
  for (uint32_t first = 0; first < n; first += (1u << 22)) {
    uint32_t cnt = std::min<uint32_t>(1u << 22, n - first);
    launch_af_samples(ds.p, t->num_samplers, cnt, first, t->seed, X.p + static_cast<size_t>(first) * AF_K1,
                      Y.p + first, nullptr, true, s);
  }
  AF_CUDA(d, cudaGetLastError());
  AF_CUDA(d, cudaMemsetAsync(m->m.grads, 0, AF_PARAMS * sizeof(float), s));
  cudaEvent_t e0, e1;
  AF_CUDA(d, cudaEventCreate(&e0));
  AF_CUDA(d, cudaEventCreate(&e1));
  AF_CUDA(d, cudaEventRecord(e0, s));
  uint32_t step = 0;
  for (uint32_t ep = 0; ep < t->epochs; ++ep)
    for (uint32_t b = 0; b < steps_per_epoch; ++b, ++step) {
      uint32_t const first = b * t->batch, cnt = std::min(t->batch, n - first);
      AF_CUDA(d, launch_af_train(m->m, X.p + static_cast<size_t>(first) * AF_K1, Y.p + first, cnt,
                                 1.0f / static_cast<float>(cnt), L.p + step, m->status,
                                 static_cast<uint32_t>(device_sms(d)), s));
      launch_af_adam(m->m, t->lr, ++m->steps, s);
      launch_af_pack(m->m, s);
    }
  AF_CUDA(d, cudaEventRecord(e1, s));
  std::vector<float> losses(steps);
  AF_CUDA(d, cudaMemcpyAsync(losses.data(), L.p, steps * sizeof(float), cudaMemcpyDeviceToHost, s));
  AF_CUDA(d, cudaStreamSynchronize(s));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rep) {
    // mean per-sample loss over the first and the last `win` batches (one
    // batch's loss is too noisy to show a trend over a short run)
    uint32_t const win = std::max(1u, std::min(16u, steps / 4));
    auto window_mean = [&](uint32_t from) {
      double sum = 0.0, cnt = 0.0;
      for (uint32_t k = from; k < from + win; ++k) {
        uint32_t const b = k % steps_per_epoch;
        sum += losses[k];
        cnt += static_cast<double>(std::min(t->batch, n - b * t->batch));
      }
      return static_cast<float>(sum / cnt);
    };
    rep->first_loss = window_mean(0);
    rep->last_loss = window_mean(steps - win);
    rep->steps = steps;
    rep->train_ms = ms;
  }
  return check_status(d, m);
}

}  // extern "C"
