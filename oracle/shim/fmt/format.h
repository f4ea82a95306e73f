// Minimal stand-in for the {fmt} calls the reference's diagnostics make
// (eflib/include/eflib/diagnostics/assert.h:45-46). Only used on error
// paths: prints the raw format string, without substitution.
#pragma once
#include <cstdio>
#include <string_view>
namespace fmt {
struct format_args_stub {};
template <typename... Args>
inline format_args_stub make_format_args(Args&&...) { return {}; }
inline void vprint(std::FILE* f, std::string_view s, format_args_stub) {
  std::fwrite(s.data(), 1, s.size(), f);
}
template <typename... Args>
inline void print(std::FILE* f, std::string_view s, Args&&...) {
  std::fwrite(s.data(), 1, s.size(), f);
  std::fputc('\n', f);
}
}  // namespace fmt
