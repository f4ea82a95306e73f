// salvia_gb300/sasl_rt.cuh -- the value types and intrinsics of SASL shaders
// translated to C++ shader bodies (sg_sasl_translate).
//
// SASL (the reference's shader language, sasl/) has HLSL's scalar, vector
// and matrix types; its code generator lowers them to LLVM vectors
// (sasl/src/codegen/cg_impl.cpp).  A translated shader uses these templates
// instead, compiled with the body for the GPU and for the host:
//
//   vec<T, N>     floatN / intN / uintN / boolN (zero-initialised)
//   mat<T, R, C>  floatRxC: R rows of C components; a uniform's words are
//                 its rows one after another, and mul(v, M) is the row
//                 vector times M, each component a left-to-right dot product
//                 of v and a column (eflib transform, math.cpp:142-154)
//
// Arithmetic is component-wise, a scalar operand applied to every component;
// the result's component type is C++'s for the component types (int with
// float gives float).  Integer division and remainder by zero give 0 rather
// than trapping on the host.  Float intrinsics call CUDA's and the C
// library's float functions (sqrtf, expf, ...), so transcendental results can
// differ between the GPU and the host in the last bits.
#pragma once

#include <cstdint>
#include <cstring>
#include <cmath>
#include <type_traits>

#include "salvia_gb300/device_shader.cuh"

#define SASL_HD __host__ __device__ inline

namespace sasl_rt {

template <class T, int N>
struct vec;
template <class T, int R, int C>
struct mat;

template <class T>
struct traits {
  using elem = T;
  static constexpr int n = 1;
};
template <class T, int N>
struct traits<vec<T, N>> {
  using elem = T;
  static constexpr int n = N;
};
template <class T, int R, int C>
struct traits<mat<T, R, C>> {
  using elem = T;
  static constexpr int n = R * C;
};
template <class T>
constexpr bool is_scalar_v = std::is_arithmetic<T>::value;

template <class T, int N>
struct vec {
  T v[N];
  SASL_HD vec() {
    for (int i = 0; i < N; ++i) v[i] = T(0);
  }
  template <class U, std::enable_if_t<std::is_arithmetic<U>::value, int> = 0>
  SASL_HD vec(U s) {  // a scalar to every component
    for (int i = 0; i < N; ++i) v[i] = static_cast<T>(s);
  }
  template <class U, int M, std::enable_if_t<(M >= N), int> = 0>
  SASL_HD vec(vec<U, M> const& o) {  // conversion, truncating to the first N components
    for (int i = 0; i < N; ++i) v[i] = static_cast<T>(o.v[i]);
  }
  SASL_HD T& operator[](int i) { return v[i]; }
  SASL_HD T const& operator[](int i) const { return v[i]; }
};

template <class T, int R, int C>
struct mat {
  vec<T, C> r[R];
  SASL_HD mat() {}
  template <class U, std::enable_if_t<std::is_arithmetic<U>::value, int> = 0>
  SASL_HD mat(U s) {
    for (int i = 0; i < R; ++i) r[i] = vec<T, C>(s);
  }
  template <class U>
  SASL_HD mat(mat<U, R, C> const& o) {
    for (int i = 0; i < R; ++i) r[i] = vec<T, C>(o.r[i]);
  }
  SASL_HD vec<T, C>& operator[](int i) { return r[i]; }
  SASL_HD vec<T, C> const& operator[](int i) const { return r[i]; }
};

// ---- division and remainder (checked for integers) --------------------------
template <class A, class B, std::enable_if_t<is_scalar_v<A> && is_scalar_v<B>, int> = 0>
SASL_HD auto div(A a, B b) {
  using R = decltype(a / b);
  if constexpr (std::is_integral<R>::value) {
    return b == B(0) ? R(0) : static_cast<R>(a / b);
  } else {
    return static_cast<R>(a) / static_cast<R>(b);
  }
}
template <class A, class B, std::enable_if_t<is_scalar_v<A> && is_scalar_v<B>, int> = 0>
SASL_HD auto mod(A a, B b) {
  using R = decltype(a + b);
  if constexpr (std::is_integral<R>::value) {
    return b == B(0) ? R(0) : static_cast<R>(a % b);
  } else {
    return static_cast<R>(fmodf(static_cast<float>(a), static_cast<float>(b)));
  }
}

// ---- component-wise operators ----------------------------------------------
#define SASL_CW_BINARY(NAME, EXPR)                                                                 \
  template <class T, class U, int N>                                                               \
  SASL_HD auto NAME(vec<T, N> const& a, vec<U, N> const& b) {                                      \
    using E = decltype(EXPR(a.v[0], b.v[0]));                                                      \
    vec<E, N> o;                                                                                   \
    for (int i = 0; i < N; ++i) o.v[i] = EXPR(a.v[i], b.v[i]);                                     \
    return o;                                                                                      \
  }                                                                                                \
  template <class T, class U, int N, std::enable_if_t<is_scalar_v<U>, int> = 0>                    \
  SASL_HD auto NAME(vec<T, N> const& a, U b) {                                                     \
    using E = decltype(EXPR(a.v[0], b));                                                           \
    vec<E, N> o;                                                                                   \
    for (int i = 0; i < N; ++i) o.v[i] = EXPR(a.v[i], b);                                          \
    return o;                                                                                      \
  }                                                                                                \
  template <class T, class U, int N, std::enable_if_t<is_scalar_v<T>, int> = 0>                    \
  SASL_HD auto NAME(T a, vec<U, N> const& b) {                                                     \
    using E = decltype(EXPR(a, b.v[0]));                                                           \
    vec<E, N> o;                                                                                   \
    for (int i = 0; i < N; ++i) o.v[i] = EXPR(a, b.v[i]);                                          \
    return o;                                                                                      \
  }                                                                                                \
  template <class T, class U, int R, int C>                                                        \
  SASL_HD auto NAME(mat<T, R, C> const& a, mat<U, R, C> const& b) {                                \
    mat<typename traits<decltype(NAME(a.r[0], b.r[0]))>::elem, R, C> o;                           \
    for (int i = 0; i < R; ++i) o.r[i] = NAME(a.r[i], b.r[i]);                                     \
    return o;                                                                                      \
  }                                                                                                \
  template <class T, class U, int R, int C, std::enable_if_t<is_scalar_v<U>, int> = 0>             \
  SASL_HD auto NAME(mat<T, R, C> const& a, U b) {                                                  \
    mat<typename traits<decltype(NAME(a.r[0], b))>::elem, R, C> o;                                 \
    for (int i = 0; i < R; ++i) o.r[i] = NAME(a.r[i], b);                                          \
    return o;                                                                                      \
  }                                                                                                \
  template <class T, class U, int R, int C, std::enable_if_t<is_scalar_v<T>, int> = 0>             \
  SASL_HD auto NAME(T a, mat<U, R, C> const& b) {                                                  \
    mat<typename traits<decltype(NAME(a, b.r[0]))>::elem, R, C> o;                                 \
    for (int i = 0; i < R; ++i) o.r[i] = NAME(a, b.r[i]);                                          \
    return o;                                                                                      \
  }

// the component operations, one function per operator
#define SASL_DEFINE_OP(FN, OP)                                                                     \
  template <class A, class B>                                                                      \
  SASL_HD auto FN(A a, B b) -> decltype(a OP b) {                                                  \
    return a OP b;                                                                                 \
  }
namespace op {
SASL_DEFINE_OP(add, +)
SASL_DEFINE_OP(sub, -)
SASL_DEFINE_OP(mul, *)
SASL_DEFINE_OP(band, &)
SASL_DEFINE_OP(bor, |)
SASL_DEFINE_OP(bxor, ^)
SASL_DEFINE_OP(shl, <<)
SASL_DEFINE_OP(shr, >>)
SASL_DEFINE_OP(lt, <)
SASL_DEFINE_OP(gt, >)
SASL_DEFINE_OP(le, <=)
SASL_DEFINE_OP(ge, >=)
SASL_DEFINE_OP(eq, ==)
SASL_DEFINE_OP(ne, !=)
SASL_DEFINE_OP(land, &&)
SASL_DEFINE_OP(lor, ||)
template <class A, class B>
SASL_HD auto sdiv(A a, B b) {
  return ::sasl_rt::div(a, b);
}
template <class A, class B>
SASL_HD auto smod(A a, B b) {
  return ::sasl_rt::mod(a, b);
}
}  // namespace op

SASL_CW_BINARY(operator+, op::add)
SASL_CW_BINARY(operator-, op::sub)
SASL_CW_BINARY(operator*, op::mul)
SASL_CW_BINARY(operator&, op::band)
SASL_CW_BINARY(operator|, op::bor)
SASL_CW_BINARY(operator^, op::bxor)
SASL_CW_BINARY(operator<<, op::shl)
SASL_CW_BINARY(operator>>, op::shr)
SASL_CW_BINARY(operator<, op::lt)
SASL_CW_BINARY(operator>, op::gt)
SASL_CW_BINARY(operator<=, op::le)
SASL_CW_BINARY(operator>=, op::ge)
SASL_CW_BINARY(operator==, op::eq)
SASL_CW_BINARY(operator!=, op::ne)
SASL_CW_BINARY(operator&&, op::land)
SASL_CW_BINARY(operator||, op::lor)
SASL_CW_BINARY(div, op::sdiv)
SASL_CW_BINARY(mod, op::smod)

template <class T, int N>
SASL_HD vec<T, N> operator-(vec<T, N> const& a) {
  vec<T, N> o;
  for (int i = 0; i < N; ++i) o.v[i] = -a.v[i];
  return o;
}
template <class T, int N>
SASL_HD vec<T, N> operator+(vec<T, N> const& a) {
  return a;
}
template <class T, int N>
SASL_HD vec<bool, N> operator!(vec<T, N> const& a) {
  vec<bool, N> o;
  for (int i = 0; i < N; ++i) o.v[i] = !a.v[i];
  return o;
}
template <class T, int N>
SASL_HD vec<T, N> operator~(vec<T, N> const& a) {
  vec<T, N> o;
  for (int i = 0; i < N; ++i) o.v[i] = ~a.v[i];
  return o;
}
template <class T, int R, int C>
SASL_HD mat<T, R, C> operator-(mat<T, R, C> const& a) {
  mat<T, R, C> o;
  for (int i = 0; i < R; ++i) o.r[i] = -a.r[i];
  return o;
}
template <class T, int R, int C>
SASL_HD mat<bool, R, C> operator!(mat<T, R, C> const& a) {
  mat<bool, R, C> o;
  for (int i = 0; i < R; ++i) o.r[i] = !a.r[i];
  return o;
}
template <class T, int R, int C>
SASL_HD mat<T, R, C> operator~(mat<T, R, C> const& a) {
  mat<T, R, C> o;
  for (int i = 0; i < R; ++i) o.r[i] = ~a.r[i];
  return o;
}

// compound assignment: the operation, then the conversion back
#define SASL_COMPOUND(OP, EXPR)                                                                    \
  template <class T, int N, class B>                                                               \
  SASL_HD vec<T, N>& operator OP(vec<T, N>& a, B const& b) {                                       \
    a = vec<T, N>(EXPR);                                                                           \
    return a;                                                                                      \
  }                                                                                                \
  template <class T, int R, int C, class B>                                                        \
  SASL_HD mat<T, R, C>& operator OP(mat<T, R, C>& a, B const& b) {                                 \
    a = mat<T, R, C>(EXPR);                                                                        \
    return a;                                                                                      \
  }
SASL_COMPOUND(+=, a + b)
SASL_COMPOUND(-=, a - b)
SASL_COMPOUND(*=, a * b)
SASL_COMPOUND(&=, a & b)
SASL_COMPOUND(|=, a | b)
SASL_COMPOUND(^=, a ^ b)
// /= and %= are emitted as a = div(a, b) and a = mod(a, b)

// ---- swizzles ---------------------------------------------------------------
template <int I, class T, int N>
SASL_HD T& comp(vec<T, N>& x) {
  static_assert(I < N, "swizzle component out of range");
  return x.v[I];
}
template <int I, class T, int N>
SASL_HD T const& comp(vec<T, N> const& x) {
  static_assert(I < N, "swizzle component out of range");
  return x.v[I];
}
template <int I, class T, std::enable_if_t<is_scalar_v<T>, int> = 0>
SASL_HD T& comp(T& s) {
  static_assert(I == 0, "swizzle component out of range");
  return s;
}
template <int I, class T, std::enable_if_t<is_scalar_v<T>, int> = 0>
SASL_HD T comp(T const& s) {
  static_assert(I == 0, "swizzle component out of range");
  return s;
}
template <int... I, class T, int N>
SASL_HD vec<T, sizeof...(I)> swz(vec<T, N> const& x) {
  vec<T, sizeof...(I)> o;
  int const idx[] = {I...};
  for (int k = 0; k < static_cast<int>(sizeof...(I)); ++k) o.v[k] = x.v[idx[k]];
  return o;
}
template <int... I, class T, std::enable_if_t<is_scalar_v<T>, int> = 0>
SASL_HD vec<T, sizeof...(I)> swz(T s) {
  return vec<T, sizeof...(I)>(s);
}
// a write mask of several components: x.yzx = r
template <int... I, class T, int N, class R>
SASL_HD void swz_set(vec<T, N>& x, R const& r) {
  int const idx[] = {I...};
  if constexpr (is_scalar_v<R>) {
    for (int k = 0; k < static_cast<int>(sizeof...(I)); ++k) x.v[idx[k]] = static_cast<T>(r);
  } else {
    for (int k = 0; k < static_cast<int>(sizeof...(I)); ++k) x.v[idx[k]] = static_cast<T>(r.v[k]);
  }
}

// ---- constructors and casts -------------------------------------------------
template <class E, class A>
SASL_HD void put(E* out, int& k, int cap, A const& a) {
  if constexpr (is_scalar_v<A>) {
    if (k < cap) out[k] = static_cast<E>(a);
    ++k;
  } else if constexpr (traits<A>::n > 0 && std::is_same<A, vec<typename traits<A>::elem, traits<A>::n>>::value) {
    for (int i = 0; i < traits<A>::n; ++i) {
      if (k < cap) out[k] = static_cast<E>(a.v[i]);
      ++k;
    }
  } else {
    for (int r = 0; r < static_cast<int>(sizeof(a.r) / sizeof(a.r[0])); ++r) put(out, k, cap, a.r[r]);
  }
}
template <class T>
SASL_HD T from_elems(typename traits<T>::elem const* e, int k) {
  T o;
  if constexpr (is_scalar_v<T>) {
    o = e[0];
  } else if constexpr (std::is_same<T, vec<typename traits<T>::elem, traits<T>::n>>::value) {
    for (int i = 0; i < traits<T>::n; ++i) o.v[i] = k == 1 ? e[0] : e[i];
  } else {
    constexpr int C = sizeof(o.r[0].v) / sizeof(o.r[0].v[0]);
    for (int i = 0; i < traits<T>::n; ++i) o.r[i / C].v[i % C] = k == 1 ? e[0] : e[i];
  }
  return o;
}
// floatN(a, b, ...) and floatRxC(...): the arguments' components in order
template <class T, class... A>
SASL_HD T make(A const&... a) {
  using E = typename traits<T>::elem;
  E buf[traits<T>::n];
  for (int i = 0; i < traits<T>::n; ++i) buf[i] = E(0);
  int k = 0;
  (put(buf, k, traits<T>::n, a), ...);
  return from_elems<T>(buf, k);
}
// (T)x: scalar to vector splats, vector to scalar takes x, vectors convert
// component-wise (truncating; missing components are 0)
template <class T, class A>
SASL_HD T cast(A const& a) {
  using E = typename traits<T>::elem;
  constexpr int n = traits<A>::n > 0 ? traits<A>::n : 1;
  E buf[n];
  int k = 0;
  put(buf, k, n, a);
  if constexpr (is_scalar_v<T>) {
    return static_cast<T>(buf[0]);
  } else {
    E full[traits<T>::n];
    for (int i = 0; i < traits<T>::n; ++i) full[i] = i < k ? buf[i] : E(0);
    return from_elems<T>(full, k == 1 ? 1 : traits<T>::n);
  }
}

// ---- registers --------------------------------------------------------------
// an interpolated register as a value of type T (its first components)
template <class T>
SASL_HD T from4(salvia_gb300::vec4 const& r) {
  using E = typename traits<T>::elem;
  E const e[4] = {static_cast<E>(r.x), static_cast<E>(r.y), static_cast<E>(r.z), static_cast<E>(r.w)};
  if constexpr (is_scalar_v<T>) {
    return e[0];
  } else {
    static_assert(traits<T>::n <= 4, "a register holds at most four components");
    T o;
    for (int i = 0; i < traits<T>::n; ++i) o.v[i] = e[i];
    return o;
  }
}
// varying register r of a pixel: selected among the registers rather than
// indexed, so that the interpolated registers stay in registers
SASL_HD salvia_gb300::vec4 varying(salvia_gb300::vs_output const& in, int r) {
  salvia_gb300::vec4 v = in.attr[0];
#pragma unroll
  for (int i = 1; i < SG_MAX_VARYINGS; ++i)
    if (r == i) v = in.attr[i];
  return v;
}
// a value written to a register: missing components are 0
template <class T>
SASL_HD salvia_gb300::vec4 to4(T const& x) {
  float e[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  if constexpr (is_scalar_v<T>) {
    e[0] = static_cast<float>(x);
  } else {
    for (int i = 0; i < traits<T>::n && i < 4; ++i) e[i] = static_cast<float>(x.v[i]);
  }
  return salvia_gb300::vec4(e[0], e[1], e[2], e[3]);
}
SASL_HD uint32_t bits(float f) {
  uint32_t u;
  memcpy(&u, &f, sizeof u);
  return u;
}
// one 32-bit uniform word into a component (floats as they are, integers by
// their bits, bools as nonzero)
template <class E>
SASL_HD E from_word(float w) {
  if constexpr (std::is_same<E, float>::value) {
    return w;
  } else if constexpr (std::is_same<E, bool>::value) {
    return bits(w) != 0u;
  } else {
    E e;
    uint32_t const u = bits(w);
    memcpy(&e, &u, sizeof e);
    return e;
  }
}

// ---- intrinsics -------------------------------------------------------------
#define SASL_UNARY_F(NAME, EXPR)                                                                   \
  SASL_HD float NAME(float x) { return EXPR; }                                                     \
  template <class T, int N>                                                                        \
  SASL_HD vec<float, N> NAME(vec<T, N> const& a) {                                                 \
    vec<float, N> o;                                                                               \
    for (int i = 0; i < N; ++i) o.v[i] = NAME(static_cast<float>(a.v[i]));                         \
    return o;                                                                                      \
  }
SASL_UNARY_F(sqrt, sqrtf(x))
SASL_UNARY_F(rsqrt, 1.0f / sqrtf(x))
SASL_UNARY_F(exp, expf(x))
SASL_UNARY_F(exp2, exp2f(x))
SASL_UNARY_F(log, logf(x))
SASL_UNARY_F(log2, log2f(x))
SASL_UNARY_F(log10, log10f(x))
SASL_UNARY_F(sin, sinf(x))
SASL_UNARY_F(cos, cosf(x))
SASL_UNARY_F(tan, tanf(x))
SASL_UNARY_F(asin, asinf(x))
SASL_UNARY_F(acos, acosf(x))
SASL_UNARY_F(atan, atanf(x))
SASL_UNARY_F(sinh, sinhf(x))
SASL_UNARY_F(cosh, coshf(x))
SASL_UNARY_F(tanh, tanhf(x))
SASL_UNARY_F(floor, floorf(x))
SASL_UNARY_F(ceil, ceilf(x))
SASL_UNARY_F(round, rintf(x))
SASL_UNARY_F(trunc, truncf(x))
SASL_UNARY_F(frac, x - floorf(x))
SASL_UNARY_F(saturate, x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x))
SASL_UNARY_F(degrees, x * 57.29577951308232f)
SASL_UNARY_F(radians, x * 0.017453292519943295f)

#define SASL_BINARY_F(NAME, EXPR)                                                                  \
  SASL_HD float NAME(float x, float y) { return EXPR; }                                            \
  template <class A, class B, std::enable_if_t<!(is_scalar_v<A> && is_scalar_v<B>), int> = 0>      \
  SASL_HD auto NAME(A const& a, B const& b) {                                                      \
    constexpr int N = traits<A>::n > traits<B>::n ? traits<A>::n : traits<B>::n;                   \
    vec<float, N> const va = cast<vec<float, N>>(a), vb = cast<vec<float, N>>(b);                  \
    vec<float, N> o;                                                                               \
    for (int i = 0; i < N; ++i) o.v[i] = NAME(va.v[i], vb.v[i]);                                   \
    return o;                                                                                      \
  }
SASL_BINARY_F(pow, powf(x, y))
SASL_BINARY_F(fmod, fmodf(x, y))
SASL_BINARY_F(atan2, atan2f(x, y))
SASL_BINARY_F(step, y >= x ? 1.0f : 0.0f)

// abs, min, max, clamp keep integer types
template <class T, std::enable_if_t<is_scalar_v<T>, int> = 0>
SASL_HD T abs(T x) {
  return x < T(0) ? T(-x) : x;
}
template <class T, int N>
SASL_HD vec<T, N> abs(vec<T, N> const& a) {
  vec<T, N> o;
  for (int i = 0; i < N; ++i) o.v[i] = abs(a.v[i]);
  return o;
}
template <class T, std::enable_if_t<is_scalar_v<T>, int> = 0>
SASL_HD T sign(T x) {
  return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0));
}
template <class T, int N>
SASL_HD vec<T, N> sign(vec<T, N> const& a) {
  vec<T, N> o;
  for (int i = 0; i < N; ++i) o.v[i] = sign(a.v[i]);
  return o;
}
template <class A, class B, std::enable_if_t<is_scalar_v<A> && is_scalar_v<B>, int> = 0>
SASL_HD auto min(A a, B b) {
  using R = decltype(a + b);
  return static_cast<R>(b) < static_cast<R>(a) ? static_cast<R>(b) : static_cast<R>(a);
}
template <class A, class B, std::enable_if_t<is_scalar_v<A> && is_scalar_v<B>, int> = 0>
SASL_HD auto max(A a, B b) {
  using R = decltype(a + b);
  return static_cast<R>(a) < static_cast<R>(b) ? static_cast<R>(b) : static_cast<R>(a);
}
template <class A, class B, std::enable_if_t<!(is_scalar_v<A> && is_scalar_v<B>), int> = 0>
SASL_HD auto min(A const& a, B const& b) {
  using E = decltype(typename traits<A>::elem() + typename traits<B>::elem());
  constexpr int N = traits<A>::n > traits<B>::n ? traits<A>::n : traits<B>::n;
  vec<E, N> const va = cast<vec<E, N>>(a), vb = cast<vec<E, N>>(b);
  vec<E, N> o;
  for (int i = 0; i < N; ++i) o.v[i] = min(va.v[i], vb.v[i]);
  return o;
}
template <class A, class B, std::enable_if_t<!(is_scalar_v<A> && is_scalar_v<B>), int> = 0>
SASL_HD auto max(A const& a, B const& b) {
  using E = decltype(typename traits<A>::elem() + typename traits<B>::elem());
  constexpr int N = traits<A>::n > traits<B>::n ? traits<A>::n : traits<B>::n;
  vec<E, N> const va = cast<vec<E, N>>(a), vb = cast<vec<E, N>>(b);
  vec<E, N> o;
  for (int i = 0; i < N; ++i) o.v[i] = max(va.v[i], vb.v[i]);
  return o;
}
template <class X, class L, class H>
SASL_HD auto clamp(X const& x, L const& lo, H const& hi) {
  return min(max(x, lo), hi);
}
// lerp(a, b, t) = a + (b - a) * t
template <class A, class B, class T>
SASL_HD auto lerp(A const& a, B const& b, T const& t) {
  return a + (b - a) * t;
}
template <class A, class B, class X>
SASL_HD auto smoothstep(A const& a, B const& b, X const& x) {
  auto const t = saturate(div(x - a, b - a));
  return t * t * (3.0f - 2.0f * t);
}

// dot products left to right (eflib dot_prod4, math.cpp:43-45)
template <class T, class U, int N>
SASL_HD auto dot(vec<T, N> const& a, vec<U, N> const& b) {
  decltype(a.v[0] * b.v[0]) s = a.v[0] * b.v[0];
  for (int i = 1; i < N; ++i) s = s + a.v[i] * b.v[i];
  return s;
}
template <class A, class B, std::enable_if_t<is_scalar_v<A> && is_scalar_v<B>, int> = 0>
SASL_HD auto dot(A a, B b) {
  return a * b;
}
template <class T>
SASL_HD vec<T, 3> cross(vec<T, 3> const& a, vec<T, 3> const& b) {
  vec<T, 3> o;
  o.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
  o.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
  o.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
  return o;
}
template <class T>
SASL_HD float length(T const& x) {
  return sqrtf(static_cast<float>(dot(x, x)));
}
template <class A, class B>
SASL_HD float distance(A const& a, B const& b) {
  return length(b - a);
}
// x / length(x)
template <class T>
SASL_HD auto normalize(T const& x) {
  return div(x, length(x));
}
// i - 2 dot(n, i) n
template <class I, class N>
SASL_HD auto reflect(I const& i, N const& n) {
  return i - (2.0f * dot(n, i)) * n;
}
template <class T, int N>
SASL_HD bool any(vec<T, N> const& a) {
  for (int i = 0; i < N; ++i)
    if (a.v[i]) return true;
  return false;
}
template <class T, int N>
SASL_HD bool all(vec<T, N> const& a) {
  for (int i = 0; i < N; ++i)
    if (!a.v[i]) return false;
  return true;
}
template <class T, std::enable_if_t<is_scalar_v<T>, int> = 0>
SASL_HD bool any(T a) {
  return a != T(0);
}
template <class T, std::enable_if_t<is_scalar_v<T>, int> = 0>
SASL_HD bool all(T a) {
  return a != T(0);
}
template <class T, int R, int C>
SASL_HD mat<T, C, R> transpose(mat<T, R, C> const& m) {
  mat<T, C, R> o;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) o.r[j].v[i] = m.r[i].v[j];
  return o;
}
// mul: row vector times matrix, matrix times column vector, matrix product;
// each component one left-to-right dot product
template <class T, class U, int R, int C>
SASL_HD auto mul(vec<T, R> const& v, mat<U, R, C> const& m) {
  vec<decltype(v.v[0] * m.r[0].v[0]), C> o;
  for (int c = 0; c < C; ++c) {
    auto s = v.v[0] * m.r[0].v[c];
    for (int r = 1; r < R; ++r) s = s + v.v[r] * m.r[r].v[c];
    o.v[c] = s;
  }
  return o;
}
template <class T, class U, int R, int C>
SASL_HD auto mul(mat<T, R, C> const& m, vec<U, C> const& v) {
  vec<decltype(m.r[0].v[0] * v.v[0]), R> o;
  for (int r = 0; r < R; ++r) o.v[r] = dot(m.r[r], v);
  return o;
}
template <class T, class U, int R, int K, int C>
SASL_HD auto mul(mat<T, R, K> const& a, mat<U, K, C> const& b) {
  mat<decltype(a.r[0].v[0] * b.r[0].v[0]), R, C> o;
  for (int r = 0; r < R; ++r) o.r[r] = mul(a.r[r], b);
  return o;
}
template <class A, class B, std::enable_if_t<is_scalar_v<A> || is_scalar_v<B>, int> = 0>
SASL_HD auto mul(A const& a, B const& b) {
  return a * b;
}
template <class T, class U, int N>
SASL_HD auto mul(vec<T, N> const& a, vec<U, N> const& b) {
  return dot(a, b);
}

}  // namespace sasl_rt
