// Stand-in for simde's SSE header. On x86-64 the native intrinsics are used
// directly; elsewhere the reference build is not supported by this shim.
#pragma once
#if defined(__x86_64__) || defined(__i386__)
#  include <xmmintrin.h>
#else
#  error "oracle/_ref is built on x86-64 only"
#endif
