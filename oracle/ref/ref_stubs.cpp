// Link stand-ins for symbols the reference's renderer.cpp names but whose
// definitions are absent from its sources at this revision (the SASL shader
// host registers tex2D* callbacks declared in namespace salvia::resource
// while sampler_api.cpp defines them in namespace salviar), and for the async
// renderer, whose bounded queue needs boost::circular_buffer.  The oracle
// drives the synchronous create_benchmark_renderer() path only, so none of
// these is ever called; each aborts if it is.
//
// ORACLE INFRASTRUCTURE -- linked only into oracle/_ref/libsalvia_ref.so.
#include <salvia/core/renderer.h>
#include <salvia/resource/sampler_api.h>

#include <cstdio>
#include <cstdlib>

namespace {
[[noreturn]] void not_used(char const* what) {
  std::fprintf(stderr, "oracle/_ref: %s is not part of the synchronous draw path\n", what);
  std::abort();
}
}  // namespace

namespace salvia::core {
renderer_ptr create_async_renderer() { not_used("create_async_renderer"); }
}  // namespace salvia::core

namespace salvia::resource {
using eflib::vec2;
using eflib::vec4;
void tex2Dlod(vec4&, sampler*, vec4&) { not_used("tex2Dlod"); }
void texCUBElod(vec4&, sampler*, vec4&) { not_used("texCUBElod"); }
void tex2Dgrad_ps(vec4*, uint32_t, sampler*, vec2*, vec2 const*, vec2 const*) {
  not_used("tex2Dgrad_ps");
}
void tex2Dbias_ps(vec4*, uint32_t, sampler*, vec4*, vec2 const*, vec2 const*) {
  not_used("tex2Dbias_ps");
}
void tex2Dlod_ps(vec4*, uint32_t, sampler*, vec4*) { not_used("tex2Dlod_ps"); }
void tex2Dproj_ps(vec4*, uint32_t, sampler*, vec4*, vec4 const*, vec4 const*) {
  not_used("tex2Dproj_ps");
}
}  // namespace salvia::resource
