// ORACLE — test infrastructure only. Nothing in the product links or calls this.
//
// HLSL vocabulary in C++17, so that the reference's compute shaders compile as C++
// and run on the CPU (the recipe in oracle/ref_build.py applies a few listed text
// rewrites first). Together with the per-pass harnesses in oracle/hlsl/passes/ this
// runs the reference's own shader text pass by pass; the oracle restatement and
// through it the GPU kernels are compared with it.
//
// Semantics follow the HLSL language where it defines them:
//   * vector types with swizzles (read, write, compound assignment), component-wise
//     operators, scalar broadcast, implicit conversion between vector types of the
//     same or a larger size (truncation), constructors from concatenated components;
//   * unsuffixed floating literals are "literal floats" (lit below): arithmetic among
//     literals and the intrinsics of literal arguments are evaluated in binary64 (as
//     DXC folds them), a literal meeting a binary32 value or an integer variable is
//     converted to binary32 first;
//   * matrices are indexed by row (m[r] is row r) and filled from column-major
//     memory (#pragma pack_matrix(column_major), frame_bindings.hlsl:2);
//   * textures: robust access (out-of-range loads return 0, stores are dropped),
//     typed views over the reference's storage formats, SampleLevel with the
//     linear-clamp sampler;
//   * compute dispatch over groups, with SV_DispatchThreadID / SV_GroupID /
//     SV_GroupThreadID / SV_GroupIndex; quad operations (QuadReadAcrossX/Y) run the
//     four lanes of a quad in lockstep on fibers.
// Where HLSL leaves a result implementation-defined, the project's numeric contract
// (oracle/omath.hpp, the same one the GPU kernels follow) defines it: exp2/exp/log2/
// sin/cos of binary32 arguments by the contract's polynomial constructions, pow(x, y)
// by repeated multiplication for y in {1, 2, 5, 2^k} and exp2(y log2 x) otherwise,
// rcp/rsqrt/normalize as divisions, f32tof16 and the storage formats' rounding,
// float->integer conversion by truncation with saturation (NaN -> 0), exact binary32
// bilinear weights.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>
#include <ucontext.h>

#include <algorithm>
#include <type_traits>
#include <utility>
#include <vector>

#include "../omath.hpp"

namespace hlsl {

using uint = uint32_t;
using dword = uint32_t;
using half = float;

// ------------------------------------------------------------------ literal floats
struct lit {
  double v;
  constexpr lit(double d) : v(d) {}
  operator float() const { return (float)v; }
};
template <class X> struct is_lit : std::false_type {};
template <> struct is_lit<lit> : std::true_type {};
template <class X> constexpr bool is_lit_v = is_lit<std::decay_t<X>>::value;

inline lit operator+(lit a, lit b) { return lit(a.v + b.v); }
inline lit operator-(lit a, lit b) { return lit(a.v - b.v); }
inline lit operator*(lit a, lit b) { return lit(a.v * b.v); }
inline lit operator/(lit a, lit b) { return lit(a.v / b.v); }
inline lit operator-(lit a) { return lit(-a.v); }
#define HLSL_LIT_MIXED(op)                                                                   \
  template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                   \
  inline auto operator op(lit a, S b) {                                                    \
    if constexpr (std::is_floating_point_v<S>) return (S)a.v op b;                         \
    else return (float)a.v op (float)b;                                                    \
  }                                                                                        \
  template <class S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                   \
  inline auto operator op(S a, lit b) {                                                    \
    if constexpr (std::is_floating_point_v<S>) return a op (S)b.v;                         \
    else return (float)a op (float)b.v;                                                    \
  }
HLSL_LIT_MIXED(+)
HLSL_LIT_MIXED(-)
HLSL_LIT_MIXED(*)
HLSL_LIT_MIXED(/)
HLSL_LIT_MIXED(<)
HLSL_LIT_MIXED(>)
HLSL_LIT_MIXED(<=)
HLSL_LIT_MIXED(>=)
HLSL_LIT_MIXED(==)
HLSL_LIT_MIXED(!=)
#undef HLSL_LIT_MIXED
inline bool operator<(lit a, lit b) { return a.v < b.v; }
inline bool operator>(lit a, lit b) { return a.v > b.v; }
template <class S> inline S& operator+=(S& a, lit b) { return a = a + b; }
template <class S> inline S& operator-=(S& a, lit b) { return a = a - b; }
template <class S> inline S& operator*=(S& a, lit b) { return a = a * b; }
template <class S> inline S& operator/=(S& a, lit b) { return a = a / b; }

// Scalar element type of a literal when it meets a vector component.
template <class X> using scal_t = std::conditional_t<is_lit_v<X>, float, std::decay_t<X>>;

// ------------------------------------------------------------------ conversions
template <class T, class U>
inline T cvt(U u) {
  if constexpr (is_lit_v<U>) {
    return cvt<T>((float)u.v);
  } else if constexpr (std::is_same_v<T, U>) {
    return u;
  } else if constexpr (std::is_same_v<T, bool>) {
    return u != U(0);
  } else if constexpr (std::is_floating_point_v<U> && std::is_same_v<T, uint32_t>) {
    return orc::to_uint((float)u);
  } else if constexpr (std::is_floating_point_v<U> && std::is_same_v<T, int32_t>) {
    return orc::to_int((float)u);
  } else {
    return static_cast<T>(u);
  }
}

// ------------------------------------------------------------------ vectors
template <class T, int N> struct vec;
template <class T, int N, int... I> struct swz;

template <class X> struct vtraits {
  static constexpr bool is_vec = false;
  static constexpr int n = 1;
  using elem = scal_t<X>;
};
template <class T, int N> struct vtraits<vec<T, N>> {
  static constexpr bool is_vec = true;
  static constexpr int n = N;
  using elem = T;
};
template <class T, int N, int... I> struct vtraits<swz<T, N, I...>> {
  static constexpr bool is_vec = true;
  static constexpr int n = (int)sizeof...(I);
  using elem = T;
};
template <class X> constexpr bool is_vec_v = vtraits<std::decay_t<X>>::is_vec;
template <class X> constexpr int n_of = vtraits<std::decay_t<X>>::n;
template <class X> using elem_t = typename vtraits<std::decay_t<X>>::elem;

template <class X>
inline elem_t<X> el(const X& x, int k) {
  if constexpr (is_vec_v<X>) return x.get(k);
  else if constexpr (is_lit_v<X>) { (void)k; return (float)x.v; }
  else { (void)k; return x; }
}

template <class T, int N, int... I>
struct swz {
  T e[N];
  static constexpr int M = (int)sizeof...(I);
  T get(int k) const {
    constexpr int idx[] = {I...};
    return e[idx[k]];
  }
  operator vec<T, M>() const { return vec<T, M>(e[I]...); }
  template <class X>
  swz& assign(const X& x) {
    constexpr int idx[] = {I...};
    T tmp[M];
    for (int k = 0; k < M; ++k) tmp[k] = cvt<T>(el(x, k));
    for (int k = 0; k < M; ++k) e[idx[k]] = tmp[k];
    return *this;
  }
  swz& operator=(const swz& o) { return assign(o); }
  template <class X>
  swz& operator=(const X& x) { return assign(x); }
#define HLSL_SWZ_COMPOUND(op)                   \
  template <class X>                            \
  swz& operator op##=(const X& x) {             \
    return assign(vec<T, M>(*this) op x);       \
  }
  HLSL_SWZ_COMPOUND(+)
  HLSL_SWZ_COMPOUND(-)
  HLSL_SWZ_COMPOUND(*)
  HLSL_SWZ_COMPOUND(/)
  HLSL_SWZ_COMPOUND(&)
  HLSL_SWZ_COMPOUND(|)
  HLSL_SWZ_COMPOUND(^)
  HLSL_SWZ_COMPOUND(<<)
  HLSL_SWZ_COMPOUND(>>)
#undef HLSL_SWZ_COMPOUND
};

template <class T, int N> struct vstore;
#include "swizzles.inc"

template <class T, int N>
struct vec : vstore<T, N> {
  using vstore<T, N>::e;
  vec() {
    for (int k = 0; k < N; ++k) e[k] = T(0);
  }
  vec(const vec& o) : vstore<T, N>() {
    for (int k = 0; k < N; ++k) e[k] = o.e[k];
  }
  vec& operator=(const vec& o) {
    for (int k = 0; k < N; ++k) e[k] = o.e[k];
    return *this;
  }
  // broadcast
  template <class S, std::enable_if_t<std::is_arithmetic_v<S> || is_lit_v<S>, int> = 0>
  vec(S s) {
    const T t = cvt<T>(s);
    for (int k = 0; k < N; ++k) e[k] = t;
  }
  // conversion from a vector of the same or a larger size
  template <class X, std::enable_if_t<is_vec_v<X> && (n_of<X> >= N) && !std::is_same_v<std::decay_t<X>, vec>, int> = 0>
  vec(const X& x) {
    for (int k = 0; k < N; ++k) e[k] = cvt<T>(el(x, k));
  }
  // concatenated components
  template <class A, class B, class... R>
  vec(const A& a, const B& b, const R&... r) {
    int k = 0;
    put(k, a);
    put(k, b);
    (put(k, r), ...);
  }
  template <class X>
  void put(int& k, const X& x) {
    for (int j = 0; j < n_of<X>; ++j) e[k++] = cvt<T>(el(x, j));
  }
  T get(int k) const { return e[k]; }
  T& operator[](int k) { return e[k]; }
  const T& operator[](int k) const { return e[k]; }
#define HLSL_VEC_COMPOUND(op)              \
  template <class X>                       \
  vec& operator op##=(const X& x) {        \
    vec r(*this op x);                     \
    return *this = r;                      \
  }
  HLSL_VEC_COMPOUND(+)
  HLSL_VEC_COMPOUND(-)
  HLSL_VEC_COMPOUND(*)
  HLSL_VEC_COMPOUND(/)
  HLSL_VEC_COMPOUND(%)
  HLSL_VEC_COMPOUND(&)
  HLSL_VEC_COMPOUND(|)
  HLSL_VEC_COMPOUND(^)
  HLSL_VEC_COMPOUND(<<)
  HLSL_VEC_COMPOUND(>>)
#undef HLSL_VEC_COMPOUND
};


template <class A, class B>
constexpr int bin_n() {
  if constexpr (is_vec_v<A> && is_vec_v<B>) return n_of<A> < n_of<B> ? n_of<A> : n_of<B>;
  else return n_of<A> > n_of<B> ? n_of<A> : n_of<B>;
}
template <class A, class B>
using enable_vec2 = std::enable_if_t<is_vec_v<A> || is_vec_v<B>, int>;

#define HLSL_VEC_BINOP(op)                                                         \
  template <class A, class B, enable_vec2<A, B> = 0>                               \
  inline auto operator op(const A& a, const B& b) {                                \
    constexpr int N = bin_n<A, B>();                                               \
    using R = decltype(std::declval<elem_t<A>>() op std::declval<elem_t<B>>());   \
    vec<R, N> r;                                                                   \
    for (int k = 0; k < N; ++k) r.e[k] = el(a, k) op el(b, k);                     \
    return r;                                                                      \
  }
HLSL_VEC_BINOP(+)
HLSL_VEC_BINOP(-)
HLSL_VEC_BINOP(*)
HLSL_VEC_BINOP(/)
HLSL_VEC_BINOP(%)
HLSL_VEC_BINOP(&)
HLSL_VEC_BINOP(|)
HLSL_VEC_BINOP(^)
HLSL_VEC_BINOP(<<)
HLSL_VEC_BINOP(>>)
#undef HLSL_VEC_BINOP

#define HLSL_VEC_CMP(op)                                      \
  template <class A, class B, enable_vec2<A, B> = 0>          \
  inline auto operator op(const A& a, const B& b) {           \
    constexpr int N = bin_n<A, B>();                          \
    vec<bool, N> r;                                           \
    for (int k = 0; k < N; ++k) r.e[k] = el(a, k) op el(b, k); \
    return r;                                                 \
  }
HLSL_VEC_CMP(<)
HLSL_VEC_CMP(>)
HLSL_VEC_CMP(<=)
HLSL_VEC_CMP(>=)
HLSL_VEC_CMP(==)
HLSL_VEC_CMP(!=)
HLSL_VEC_CMP(&&)
HLSL_VEC_CMP(||)
#undef HLSL_VEC_CMP

template <class A, std::enable_if_t<is_vec_v<A>, int> = 0>
inline auto operator-(const A& a) {
  vec<elem_t<A>, n_of<A>> r;
  for (int k = 0; k < n_of<A>; ++k) r.e[k] = -el(a, k);
  return r;
}
template <class A, std::enable_if_t<is_vec_v<A>, int> = 0>
inline auto operator!(const A& a) {
  vec<bool, n_of<A>> r;
  for (int k = 0; k < n_of<A>; ++k) r.e[k] = !el(a, k);
  return r;
}
template <class A, std::enable_if_t<is_vec_v<A>, int> = 0>
inline auto operator~(const A& a) {
  vec<elem_t<A>, n_of<A>> r;
  for (int k = 0; k < n_of<A>; ++k) r.e[k] = ~el(a, k);
  return r;
}

using float2 = vec<float, 2>;
using float3 = vec<float, 3>;
using float4 = vec<float, 4>;
using int2 = vec<int32_t, 2>;
using int3 = vec<int32_t, 3>;
using int4 = vec<int32_t, 4>;
using uint2 = vec<uint32_t, 2>;
using uint3 = vec<uint32_t, 3>;
using uint4 = vec<uint32_t, 4>;
using bool2 = vec<bool, 2>;
using bool3 = vec<bool, 3>;
using bool4 = vec<bool, 4>;
using half2 = float2;
using half3 = float3;
using half4 = float4;

// `.xx` / `.xxx` of a scalar (or a vector's first component), as rewritten by the recipe.
template <int N, class X>
inline vec<elem_t<X>, N> splat(const X& x) {
  return vec<elem_t<X>, N>(el(x, 0));
}

// ------------------------------------------------------------------ matrices
template <int R, int C>
struct mat {
  vec<float, C> m[R];  // rows
  mat() = default;
  // Components in row-major order (scalars or vectors), as HLSL's constructor.
  template <class A, class... Rest>
  explicit mat(const A& a, const Rest&... rest) {
    int k = 0;
    put(k, a);
    (put(k, rest), ...);
  }
  template <class X>
  void put(int& k, const X& x) {
    for (int j = 0; j < n_of<X>; ++j, ++k) m[k / C].e[k % C] = cvt<float>(el(x, j));
  }
  vec<float, C>& operator[](int r) { return m[r]; }
  const vec<float, C>& operator[](int r) const { return m[r]; }
  static mat from_column_major(const float* p) {
    mat o;
    for (int c = 0; c < C; ++c)
      for (int r = 0; r < R; ++r) o.m[r].e[c] = p[c * R + r];
    return o;
  }
};
using float2x2 = mat<2, 2>;
using float3x3 = mat<3, 3>;
using float4x4 = mat<4, 4>;

// ------------------------------------------------------------------ scalar helpers
template <class X>
using fscal = std::conditional_t<is_lit_v<X>, float, X>;

// Elementwise application of a unary function to a scalar or a vector.
template <class X, class F>
inline auto map1(const X& x, F f) {
  if constexpr (is_vec_v<X>) {
    using R = decltype(f(el(x, 0)));
    vec<R, n_of<X>> r;
    for (int k = 0; k < n_of<X>; ++k) r.e[k] = f(el(x, k));
    return r;
  } else {
    return f(x);
  }
}
template <class A, class B, class F>
inline auto map2(const A& a, const B& b, F f) {
  if constexpr (is_vec_v<A> || is_vec_v<B>) {
    constexpr int N = bin_n<A, B>();
    using R = decltype(f(el(a, 0), el(b, 0)));
    vec<R, N> r;
    for (int k = 0; k < N; ++k) r.e[k] = f(el(a, k), el(b, k));
    return r;
  } else {
    return f(a, b);
  }
}
template <class A, class B, class C, class F>
inline auto map3(const A& a, const B& b, const C& c, F f) {
  if constexpr (is_vec_v<A> || is_vec_v<B> || is_vec_v<C>) {
    constexpr int N1 = bin_n<A, B>();
    constexpr int N = N1 > n_of<C> ? N1 : n_of<C>;
    using R = decltype(f(el(a, 0), el(b, 0), el(c, 0)));
    vec<R, N> r;
    for (int k = 0; k < N; ++k) r.e[k] = f(el(a, k), el(b, k), el(c, k));
    return r;
  } else {
    return f(a, b, c);
  }
}

// HLSL promotion of two scalars (a literal takes the other operand's type).
template <class A, class B>
using prom_t = decltype(std::declval<scal_t<A>>() + std::declval<scal_t<B>>());

// ------------------------------------------------------------------ intrinsics
// Transcendentals: literal arguments are folded in binary64 (libm); binary32
// arguments use the contract's constructions.
inline lit exp(lit x) { return lit(::exp(x.v)); }
inline lit exp2(lit x) { return lit(::exp2(x.v)); }
inline lit log(lit x) { return lit(::log(x.v)); }
inline lit log2(lit x) { return lit(::log2(x.v)); }
inline lit sin(lit x) { return lit(::sin(x.v)); }
inline lit cos(lit x) { return lit(::cos(x.v)); }
inline lit sqrt(lit x) { return lit(::sqrt(x.v)); }
inline float exp2_f(float x) { return orc::exp2_own(x); }
inline float exp_f(float x) { return orc::exp_own(x); }
inline float log2_f(float x) { return orc::log2_own(x); }
inline float log_f(float x) { return orc::log2_own(x) * 0.693147182464599609375f; }
template <class X, std::enable_if_t<!is_lit_v<X>, int> = 0>
inline auto exp2(const X& x) { return map1(x, [](float v) { return exp2_f(v); }); }
template <class X, std::enable_if_t<!is_lit_v<X>, int> = 0>
inline auto exp(const X& x) { return map1(x, [](float v) { return exp_f(v); }); }
template <class X, std::enable_if_t<!is_lit_v<X>, int> = 0>
inline auto log2(const X& x) { return map1(x, [](float v) { return log2_f(v); }); }
template <class X, std::enable_if_t<!is_lit_v<X>, int> = 0>
inline auto log(const X& x) { return map1(x, [](float v) { return log_f(v); }); }
template <class X, std::enable_if_t<!is_lit_v<X>, int> = 0>
inline auto sin(const X& x) { return map1(x, [](float v) { return orc::sin_own(v); }); }
template <class X, std::enable_if_t<!is_lit_v<X>, int> = 0>
inline auto cos(const X& x) { return map1(x, [](float v) { return orc::cos_own(v); }); }
template <class X, class S, class C>
inline void sincos(const X& x, S& s, C& c) {
  s = sin(x);
  c = cos(x);
}
template <class X, std::enable_if_t<!is_lit_v<X>, int> = 0>
inline auto sqrt(const X& x) { return map1(x, [](float v) { return sqrtf(v); }); }
template <class X>
inline auto rsqrt(const X& x) { return map1(x, [](float v) { return 1.0f / sqrtf(v); }); }
template <class X>
inline auto rcp(const X& x) { return map1(x, [](float v) { return 1.0f / v; }); }
template <class X>
inline auto floor(const X& x) { return map1(x, [](float v) { return floorf(v); }); }
template <class X>
inline auto ceil(const X& x) { return map1(x, [](float v) { return ceilf(v); }); }
template <class X>
inline auto round(const X& x) { return map1(x, [](float v) { return rintf(v); }); }
template <class X>
inline auto frac(const X& x) { return map1(x, [](float v) { return v - floorf(v); }); }
template <class X>
inline auto saturate(const X& x) { return map1(x, [](float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }); }
template <class X>
inline auto isnan(const X& x) { return map1(x, [](float v) { return orc::isnan_(v); }); }
template <class X>
inline auto sign(const X& x) {
  return map1(x, [](auto v) -> int32_t { return v > 0 ? 1 : (v < 0 ? -1 : 0); });
}
template <class X>
inline auto abs(const X& x) {
  return map1(x, [](auto v) {
    using V = decltype(v);
    if constexpr (std::is_floating_point_v<V>) return fabsf(v);
    else if constexpr (std::is_signed_v<V>) return v < 0 ? -v : v;
    else return v;
  });
}
inline lit abs(lit x) { return lit(::fabs(x.v)); }

template <class A, class B>
inline auto max(const A& a, const B& b) {
  if constexpr (is_lit_v<A> && is_lit_v<B>) return lit(a.v > b.v ? a.v : b.v);
  else
    return map2(a, b, [](auto x, auto y) {
      using R = prom_t<decltype(x), decltype(y)>;
      if constexpr (std::is_floating_point_v<R>) return fmaxf((float)x, (float)y);
      else return (R)x > (R)y ? (R)x : (R)y;
    });
}
template <class A, class B>
inline auto min(const A& a, const B& b) {
  if constexpr (is_lit_v<A> && is_lit_v<B>) return lit(a.v < b.v ? a.v : b.v);
  else
    return map2(a, b, [](auto x, auto y) {
      using R = prom_t<decltype(x), decltype(y)>;
      if constexpr (std::is_floating_point_v<R>) return fminf((float)x, (float)y);
      else return (R)x < (R)y ? (R)x : (R)y;
    });
}
template <class X, class A, class B>
inline auto clamp(const X& x, const A& a, const B& b) {
  return min(max(x, a), b);
}
template <class A, class B, class S>
inline auto lerp(const A& a, const B& b, const S& s) {
  return map3(a, b, s, [](float x, float y, float t) { return x + t * (y - x); });
}
template <class A, class B>
inline auto step(const A& a, const B& b) {
  return map2(a, b, [](float y, float x) { return x >= y ? 1.0f : 0.0f; });
}
template <class A, class B, class C>
inline auto smoothstep(const A& a, const B& b, const C& x) {
  return map3(a, b, x, [](float lo, float hi, float v) {
    float t = fminf(fmaxf((v - lo) / (hi - lo), 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
  });
}
// pow: repeated multiplication for the exponents the contract lists, else exp2(y log2 x).
inline float pow_f(float x, float y) {
  if (y == 1.0f) return x;
  if (y == 2.0f) return x * x;
  if (y == 5.0f) return orc::pow5(x);
  for (int k = 2; k <= 10; ++k)
    if (y == (float)(1 << k)) {
      float r = x;
      for (int i = 0; i < k; ++i) r = r * r;
      return r;
    }
  return orc::exp2_own(y * orc::log2_own(x));
}
template <class A, class B>
inline auto pow(const A& a, const B& b) {
  if constexpr (is_lit_v<A> && is_lit_v<B>) return lit(::pow(a.v, b.v));
  else return map2(a, b, [](float x, float y) { return pow_f(x, y); });
}
template <class A, class B>
inline auto fmod(const A& a, const B& b) {
  return map2(a, b, [](float x, float y) { return fmodf(x, y); });
}
template <class A, class B, std::enable_if_t<is_vec_v<A> || is_vec_v<B>, int> = 0>
inline auto dot(const A& a, const B& b) {
  constexpr int N = bin_n<A, B>();
  using R = decltype(std::declval<elem_t<A>>() * std::declval<elem_t<B>>());
  R s = el(a, 0) * el(b, 0);
  for (int k = 1; k < N; ++k) s = s + el(a, k) * el(b, k);
  return s;
}
template <class A>
inline float length(const A& a) { return sqrtf(dot(a, a)); }
template <class A, class B>
inline float distance(const A& a, const B& b) { return length(a - b); }
template <class A>
inline auto normalize(const A& a) {
  const float r = 1.0f / sqrtf(dot(a, a));
  return vec<float, n_of<A>>(a) * r;
}
template <class A, class B>
inline float3 cross(const A& a, const B& b) {
  const float3 x(a), y(b);
  return float3(x.e[1] * y.e[2] - x.e[2] * y.e[1], x.e[2] * y.e[0] - x.e[0] * y.e[2],
                x.e[0] * y.e[1] - x.e[1] * y.e[0]);
}
template <class A, class B>
inline auto reflect(const A& i, const B& n) {
  return vec<float, n_of<A>>(i) - 2.0f * dot(n, i) * vec<float, n_of<A>>(n);
}
template <class A>
inline bool all(const A& a) {
  for (int k = 0; k < n_of<A>; ++k)
    if (!el(a, k)) return false;
  return true;
}
template <class A>
inline bool any(const A& a) {
  for (int k = 0; k < n_of<A>; ++k)
    if (el(a, k)) return true;
  return false;
}
template <class C, class A, class B>
inline auto select(const C& c, const A& a, const B& b) {
  return map3(c, a, b, [](bool t, auto x, auto y) {
    using R = prom_t<decltype(x), decltype(y)>;
    return t ? (R)x : (R)y;
  });
}
template <class X>
inline auto asuint(const X& x) {
  return map1(x, [](auto v) -> uint32_t {
    if constexpr (std::is_floating_point_v<decltype(v)>) return orc::asuint((float)v);
    else return (uint32_t)v;
  });
}
template <class X>
inline auto asint(const X& x) {
  return map1(x, [](auto v) -> int32_t {
    if constexpr (std::is_floating_point_v<decltype(v)>) return (int32_t)orc::asuint((float)v);
    else return (int32_t)v;
  });
}
template <class X>
inline auto asfloat(const X& x) {
  return map1(x, [](auto v) -> float {
    if constexpr (std::is_floating_point_v<decltype(v)>) return (float)v;
    else return orc::asfloat((uint32_t)v);
  });
}
template <class X>
inline auto f32tof16(const X& x) { return map1(x, [](float v) { return orc::f32tof16(v); }); }
template <class X>
inline auto f16tof32(const X& x) { return map1(x, [](uint32_t v) { return orc::f16tof32(v & 0xFFFFu); }); }
template <class X>
inline auto firstbithigh(const X& x) {
  return map1(x, [](uint32_t v) -> uint32_t { return v ? 31u - (uint32_t)__builtin_clz(v) : 0xFFFFFFFFu; });
}
template <class X>
inline auto firstbitlow(const X& x) {
  return map1(x, [](uint32_t v) -> uint32_t { return v ? (uint32_t)__builtin_ctz(v) : 0xFFFFFFFFu; });
}
template <class X>
inline auto countbits(const X& x) {
  return map1(x, [](uint32_t v) -> uint32_t { return (uint32_t)__builtin_popcount(v); });
}
template <class X>
inline auto reversebits(const X& x) {
  return map1(x, [](uint32_t v) -> uint32_t {
    uint32_t r = 0;
    for (int k = 0; k < 32; ++k) r |= ((v >> k) & 1u) << (31 - k);
    return r;
  });
}

// mul(M, v) = rows of M dotted with v; mul(v, M) = v combined with M's rows.
template <int R, int C, class V, std::enable_if_t<is_vec_v<V>, int> = 0>
inline vec<float, R> mul(const mat<R, C>& m, const V& v) {
  vec<float, R> r;
  for (int i = 0; i < R; ++i) r.e[i] = dot(m.m[i], vec<float, C>(v));
  return r;
}
template <int R, int C, class V, std::enable_if_t<is_vec_v<V>, int> = 0>
inline vec<float, C> mul(const V& v, const mat<R, C>& m) {
  vec<float, C> r;
  const vec<float, R> x(v);
  for (int j = 0; j < C; ++j) {
    float s = x.e[0] * m.m[0].e[j];
    for (int i = 1; i < R; ++i) s = s + x.e[i] * m.m[i].e[j];
    r.e[j] = s;
  }
  return r;
}
template <int R, int C>
inline mat<C, R> transpose(const mat<R, C>& m) {
  mat<C, R> o;
  for (int r = 0; r < R; ++r)
    for (int c = 0; c < C; ++c) o.m[c].e[r] = m.m[r].e[c];
  return o;
}

// Scalar casts written as functional casts in the shaders (`uint(x)`, `int(x)`,
// `float(x)`, `bool(x)`), rewritten by the recipe to hlsl::cast<T>(x).
template <class T, class X>
inline T cast(const X& x) {
  if constexpr (is_vec_v<X>) return cvt<T>(el(x, 0));
  else return cvt<T>(x);
}

// ------------------------------------------------------------------ atomics
// Dispatches run one thread at a time, so the interlocked operations are plain
// read-modify-writes.
template <class D, class V>
inline void InterlockedAdd(D& d, V v) { d = d + (D)v; }
template <class D, class V, class O>
inline void InterlockedAdd(D& d, V v, O& orig) { orig = d; d = d + (D)v; }
template <class D, class V>
inline void InterlockedMax(D& d, V v) { if ((D)v > d) d = (D)v; }
template <class D, class V, class O>
inline void InterlockedMax(D& d, V v, O& orig) { orig = d; if ((D)v > d) d = (D)v; }
template <class D, class V>
inline void InterlockedMin(D& d, V v) { if ((D)v < d) d = (D)v; }
template <class D, class V>
inline void InterlockedOr(D& d, V v) { d = d | (D)v; }
template <class D, class V>
inline void InterlockedAnd(D& d, V v) { d = d & (D)v; }
template <class D, class C, class V, class O>
inline void InterlockedCompareExchange(D& d, C cmp, V v, O& orig) {
  orig = d;
  if (d == (D)cmp) d = (D)v;
}
template <class D, class V, class O>
inline void InterlockedExchange(D& d, V v, O& orig) { orig = d; d = (D)v; }

// ------------------------------------------------------------------ storage formats
enum Fmt : int {
  FMT_R32F, FMT_RG32F, FMT_RGBA32F, FMT_R32UI, FMT_RG32UI, FMT_RGBA32UI,
  FMT_R11G11B10F, FMT_R16F, FMT_RG16F, FMT_RGBA16F, FMT_R8UNORM, FMT_RGBA8UNORM,
  // An RGBA16F texture whose y and z channels are always 0, stored as its x and a
  // halves (the AO history records).
  FMT_XA16F
};
inline int fmt_bytes(Fmt f) {
  switch (f) {
    case FMT_R32F: case FMT_R32UI: case FMT_R11G11B10F: case FMT_RG16F: case FMT_RGBA8UNORM: case FMT_XA16F:
      return 4;
    case FMT_RG32F: case FMT_RG32UI: case FMT_RGBA16F: return 8;
    case FMT_RGBA32F: case FMT_RGBA32UI: return 16;
    case FMT_R16F: return 2;
    case FMT_R8UNORM: return 1;
  }
  return 4;
}
inline bool fmt_is_uint(Fmt f) { return f == FMT_R32UI || f == FMT_RG32UI || f == FMT_RGBA32UI; }
inline int fmt_comps(Fmt f) {
  switch (f) {
    case FMT_R32F: case FMT_R32UI: case FMT_R16F: case FMT_R8UNORM: return 1;
    case FMT_RG32F: case FMT_RG32UI: case FMT_RG16F: return 2;
    case FMT_R11G11B10F: return 3;
    default: return 4;
  }
}

// One image: `layers` planes of w*h texels in the format, row-major, layer-planar.
// A texel may sit inside a larger per-pixel record: `stride` bytes between texels
// (0: the format's size) and `offset` bytes into the record.
struct Image {
  void* data = nullptr;
  int w = 0, h = 0, layers = 1;
  Fmt fmt = FMT_R32F;
  int stride = 0, offset = 0;
  uint8_t* texel(int x, int y, int layer) const {
    const size_t st = stride ? (size_t)stride : (size_t)fmt_bytes(fmt);
    return (uint8_t*)data + ((size_t)layer * w * h + (size_t)y * w + x) * st + offset;
  }
  bool in(int x, int y, int layer) const {
    return data && x >= 0 && y >= 0 && x < w && y < h && layer >= 0 && layer < layers;
  }
  // Float formats: the stored components as binary32 (missing ones 0, alpha 1).
  float4 load_f(int x, int y, int layer) const {
    float4 r(0.0f, 0.0f, 0.0f, 1.0f);
    if (!in(x, y, layer)) return float4(0.0f);
    const uint8_t* p = texel(x, y, layer);
    switch (fmt) {
      case FMT_R32F: case FMT_RG32F: case FMT_RGBA32F: {
        float v[4];
        memcpy(v, p, 4 * fmt_comps(fmt));
        for (int k = 0; k < fmt_comps(fmt); ++k) r.e[k] = v[k];
        break;
      }
      case FMT_R11G11B10F: {
        uint32_t u;
        memcpy(&u, p, 4);
        orc::float3 c = orc::load_r11g11b10(u);
        r = float4(c.x, c.y, c.z, 1.0f);
        break;
      }
      case FMT_R16F: case FMT_RG16F: case FMT_RGBA16F: {
        uint16_t v[4];
        memcpy(v, p, 2 * fmt_comps(fmt));
        for (int k = 0; k < fmt_comps(fmt); ++k) r.e[k] = orc::f16tof32(v[k]);
        break;
      }
      case FMT_R8UNORM: r.e[0] = orc::load_unorm8(p[0]); break;
      case FMT_RGBA8UNORM:
        for (int k = 0; k < 4; ++k) r.e[k] = orc::load_unorm8(p[k]);
        break;
      case FMT_XA16F: {
        uint16_t v[2];
        memcpy(v, p, 4);
        r = float4(orc::f16tof32(v[0]), 0.0f, 0.0f, orc::f16tof32(v[1]));
        break;
      }
      default: break;
    }
    return r;
  }
  uint4 load_u(int x, int y, int layer) const {
    uint4 r(0u);
    if (!in(x, y, layer)) return r;
    uint32_t v[4] = {0, 0, 0, 0};
    memcpy(v, texel(x, y, layer), fmt_bytes(fmt));
    for (int k = 0; k < 4; ++k) r.e[k] = v[k];
    return r;
  }
  void store_f(int x, int y, int layer, float4 c) const {
    if (!in(x, y, layer)) return;
    uint8_t* p = texel(x, y, layer);
    switch (fmt) {
      case FMT_R32F: case FMT_RG32F: case FMT_RGBA32F: {
        float v[4] = {c.e[0], c.e[1], c.e[2], c.e[3]};
        memcpy(p, v, 4 * fmt_comps(fmt));
        break;
      }
      case FMT_R11G11B10F: {
        uint32_t u = orc::store_r11g11b10(orc::F3(c.e[0], c.e[1], c.e[2]));
        memcpy(p, &u, 4);
        break;
      }
      case FMT_R16F: case FMT_RG16F: case FMT_RGBA16F: {
        uint16_t v[4];
        for (int k = 0; k < 4; ++k) v[k] = (uint16_t)orc::f32tof16(c.e[k]);
        memcpy(p, v, 2 * fmt_comps(fmt));
        break;
      }
      case FMT_R8UNORM: p[0] = orc::store_unorm8(c.e[0]); break;
      case FMT_RGBA8UNORM:
        for (int k = 0; k < 4; ++k) p[k] = orc::store_unorm8(c.e[k]);
        break;
      case FMT_XA16F: {
        uint16_t v[2] = {(uint16_t)orc::f32tof16(c.e[0]), (uint16_t)orc::f32tof16(c.e[3])};
        memcpy(p, v, 4);
        break;
      }
      default: break;
    }
  }
  void store_u(int x, int y, int layer, uint4 v) const {
    if (!in(x, y, layer)) return;
    uint32_t a[4] = {v.e[0], v.e[1], v.e[2], v.e[3]};
    memcpy(texel(x, y, layer), a, fmt_bytes(fmt));
  }
};

template <class T>
inline T from_texel(const Image& im, int x, int y, int layer) {
  if (fmt_is_uint(im.fmt)) return T(uint4(im.load_u(x, y, layer)));
  return T(im.load_f(x, y, layer));
}
template <class T>
inline void to_texel(const Image& im, int x, int y, int layer, const T& v) {
  if (fmt_is_uint(im.fmt)) im.store_u(x, y, layer, uint4(vec<uint32_t, 4>(v, 0u, 0u, 0u)));
  else im.store_f(x, y, layer, float4(vec<float, 4>(v, 0.0f, 0.0f, 0.0f)));
}
// T may be a scalar or a vector; pad to 4 components for the texel routines.
template <class T>
inline vec<elem_t<T>, 4> pad4(const T& v) {
  vec<elem_t<T>, 4> r(0);
  for (int k = 0; k < n_of<T>; ++k) r.e[k] = el(v, k);
  return r;
}
template <class T>
inline T texel_load(const Image& im, int x, int y, int layer) {
  vec<float, 4> f = fmt_is_uint(im.fmt) ? vec<float, 4>(0.0f) : im.load_f(x, y, layer);
  uint4 u = fmt_is_uint(im.fmt) ? im.load_u(x, y, layer) : uint4(0u);
  if constexpr (is_vec_v<T>) {
    T r;
    for (int k = 0; k < n_of<T>; ++k)
      r.e[k] = fmt_is_uint(im.fmt) ? cvt<elem_t<T>>(u.e[k]) : cvt<elem_t<T>>(f.e[k]);
    return r;
  } else {
    return fmt_is_uint(im.fmt) ? cvt<T>(u.e[0]) : cvt<T>(f.e[0]);
  }
}
template <class T>
inline void texel_store(const Image& im, int x, int y, int layer, const T& v) {
  if (fmt_is_uint(im.fmt)) {
    uint4 u(0u);
    for (int k = 0; k < n_of<T>; ++k) u.e[k] = cvt<uint32_t>(el(v, k));
    im.store_u(x, y, layer, u);
  } else {
    float4 f(0.0f);
    for (int k = 0; k < n_of<T>; ++k) f.e[k] = cvt<float>(el(v, k));
    im.store_f(x, y, layer, f);
  }
}

struct SamplerState {};

template <class T>
struct Texture2D {
  Image img;
  template <class C>
  T operator[](const C& c) const {
    return texel_load<T>(img, cvt<int32_t>(el(c, 0)), cvt<int32_t>(el(c, 1)), 0);
  }
  template <class C>
  T Load(const C& c) const {  // int3(x, y, mip)
    return texel_load<T>(img, el(c, 0), el(c, 1), 0);
  }
  void GetDimensions(uint32_t& w, uint32_t& h) const {
    w = (uint32_t)img.w;
    h = (uint32_t)img.h;
  }
  void GetDimensions(uint32_t mip, uint32_t& w, uint32_t& h, uint32_t& levels) const {
    (void)mip;
    w = (uint32_t)img.w;
    h = (uint32_t)img.h;
    levels = 1;
  }
  // SampleLevel with a linear-clamp sampler at mip 0: exact binary32 bilinear.
  template <class UV, class L>
  T SampleLevel(const SamplerState&, const UV& uv, const L&) const {
    const float sx = el(uv, 0) * (float)img.w - 0.5f, sy = el(uv, 1) * (float)img.h - 0.5f;
    const float bx = floorf(sx), by = floorf(sy);
    const float fx = sx - bx, fy = sy - by;
    const int ix = orc::to_int(bx), iy = orc::to_int(by);
    const int x0 = std::min(std::max(ix, 0), img.w - 1), x1 = std::min(std::max(ix + 1, 0), img.w - 1);
    const int y0 = std::min(std::max(iy, 0), img.h - 1), y1 = std::min(std::max(iy + 1, 0), img.h - 1);
    const float4 a = img.load_f(x0, y0, 0), b = img.load_f(x1, y0, 0), c = img.load_f(x0, y1, 0),
                 d = img.load_f(x1, y1, 0);
    float4 r;
    for (int k = 0; k < 4; ++k) {
      const float top = a.e[k] + fx * (b.e[k] - a.e[k]);
      const float bot = c.e[k] + fx * (d.e[k] - c.e[k]);
      r.e[k] = top + fy * (bot - top);
    }
    if constexpr (is_vec_v<T>) return T(r);
    else return r.e[0];
  }
};

// Element of an RW texture: reads load the texel (for vector texels the reference
// also carries the loaded value, so that `rw[id].xyz` reads work), assignments store.
struct TexScalarBase {};
template <class T>
struct TexRef : std::conditional_t<is_vec_v<T>, T, TexScalarBase> {
  using Base = std::conditional_t<is_vec_v<T>, T, TexScalarBase>;
  const Image* img;
  int x, y;
  TexRef(const Image* im, int px, int py) : img(im), x(px), y(py) {
    if constexpr (is_vec_v<T>) static_cast<T&>(*this) = texel_load<T>(*img, x, y, 0);
  }
  TexRef(const TexRef& o) : Base(o), img(o.img), x(o.x), y(o.y) {}
  operator T() const { return texel_load<T>(*img, x, y, 0); }
  template <class X>
  TexRef& operator=(const X& v) {
    const T t(v);
    texel_store<T>(*img, x, y, 0, t);
    if constexpr (is_vec_v<T>) static_cast<T&>(*this) = t;
    return *this;
  }
  TexRef& operator=(const TexRef& o) { return *this = (T)o; }
#define HLSL_TEXREF_COMPOUND(op)                 \
  template <class X>                             \
  TexRef& operator op##=(const X& v) {           \
    return *this = T((T)(*this) op v);           \
  }
  HLSL_TEXREF_COMPOUND(+)
  HLSL_TEXREF_COMPOUND(-)
  HLSL_TEXREF_COMPOUND(*)
#undef HLSL_TEXREF_COMPOUND
};
template <class T>
struct vtraits<TexRef<T>> : vtraits<T> {};

template <class T>
struct RWTexture2D {
  Image img;
  template <class C>
  TexRef<T> operator[](const C& c) const {
    return TexRef<T>(&img, cvt<int32_t>(el(c, 0)), cvt<int32_t>(el(c, 1)));
  }
  void GetDimensions(uint32_t& w, uint32_t& h) const {
    w = (uint32_t)img.w;
    h = (uint32_t)img.h;
  }
};

template <class T>
struct Texture2DArray {
  Image img;
  template <class C>
  T operator[](const C& c) const {
    return texel_load<T>(img, cvt<int32_t>(el(c, 0)), cvt<int32_t>(el(c, 1)), cvt<int32_t>(el(c, 2)));
  }
  void GetDimensions(uint32_t mip, uint32_t& w, uint32_t& h, uint32_t& elements, uint32_t& levels) const {
    (void)mip;
    w = (uint32_t)img.w;
    h = (uint32_t)img.h;
    elements = (uint32_t)img.layers;
    levels = 1;
  }
};

template <class T>
struct StructuredBuffer {
  const T* data = nullptr;
  uint32_t count = 0;
  T operator[](uint32_t i) const { return i < count ? data[i] : T{}; }
  void GetDimensions(uint32_t& n, uint32_t& stride) const {
    n = count;
    stride = (uint32_t)sizeof(T);
  }
};
template <class T>
struct RWStructuredBuffer {
  T* data = nullptr;
  uint32_t count = 0;
  T& operator[](uint32_t i) const {
    static thread_local T sink;
    if (i < count) return data[i];
    sink = T{};
    return sink;
  }
  void GetDimensions(uint32_t& n, uint32_t& stride) const {
    n = count;
    stride = (uint32_t)sizeof(T);
  }
};
struct RWByteAddressBuffer {
  uint8_t* data = nullptr;
  uint32_t bytes = 0;
  uint32_t Load(uint32_t addr) const {
    addr &= ~3u;
    uint32_t v = 0;
    if (addr + 4 <= bytes) memcpy(&v, data + addr, 4);
    return v;
  }
  void Store(uint32_t addr, uint32_t v) const {
    addr &= ~3u;
    if (addr + 4 <= bytes) memcpy(data + addr, &v, 4);
  }
};

template <class T>
struct ConstantBuffer : T {};

// ------------------------------------------------------------------ dispatch
struct ThreadIds {
  uint3 dispatch_thread_id, group_id, group_thread_id;
  uint32_t group_index;
};
template <class P, class V>
inline P thread_param(const V& v) {
  if constexpr (is_vec_v<P>) return P(v);
  else return cvt<P>(el(v, 0));
}
inline uint32_t thread_param_index(uint32_t i) { return i; }

// Quad lockstep: each group's threads run as fibers; QuadReadAcross* deposits the
// lane's value, lets the other lanes of its quad (lanes 4q..4q+3 of the group) reach
// the same call, and reads the partner's.
struct FiberGroup;
struct Fiber {
  ucontext_t ctx;
  std::vector<char> stack;
  bool done = false;
  int lane = 0;
  FiberGroup* group = nullptr;
  ThreadIds ids;
};
struct FiberGroup {
  ucontext_t sched;
  std::vector<Fiber> fibers;
  int current = -1;
  struct QuadSlot {
    float4 v[4];
    int arrived = 0, left = 0;
  };
  std::vector<QuadSlot> quads;
  void (*entry)(const ThreadIds&) = nullptr;
};
inline FiberGroup*& cur_group() {
  static thread_local FiberGroup* g = nullptr;
  return g;
}
inline void fiber_yield() {
  FiberGroup* g = cur_group();
  Fiber& f = g->fibers[g->current];
  swapcontext(&f.ctx, &g->sched);
}
inline void fiber_trampoline(unsigned lo, unsigned hi) {
  Fiber* f = (Fiber*)(((uintptr_t)hi << 32) | (uintptr_t)lo);
  f->group->entry(f->ids);
  f->done = true;
  swapcontext(&f->ctx, &f->group->sched);
}
template <class T>
inline T quad_read(const T& v, int lane_xor) {
  FiberGroup* g = cur_group();
  Fiber& f = g->fibers[g->current];
  FiberGroup::QuadSlot& q = g->quads[f.lane >> 2];
  const int me = f.lane & 3, base = f.lane & ~3;
  auto live = [&]() {
    int n = 0;
    for (int k = 0; k < 4; ++k)
      if (base + k < (int)g->fibers.size() && !g->fibers[base + k].done) ++n;
    return n;
  };
  while (q.left != 0) fiber_yield();
  q.v[me] = float4(pad4(v));
  ++q.arrived;
  while (q.arrived < live()) fiber_yield();
  T r;
  if constexpr (is_vec_v<T>) r = T(q.v[me ^ lane_xor]);
  else r = cvt<T>(q.v[me ^ lane_xor].e[0]);
  if (++q.left >= live()) {
    q.arrived = 0;  // the last reader of this exchange resets the slot
    q.left = 0;
  } else {
    while (q.left != 0) fiber_yield();
  }
  return r;
}
template <class T>
inline T QuadReadAcrossX(const T& v) { return quad_read(v, 1); }
template <class T>
inline T QuadReadAcrossY(const T& v) { return quad_read(v, 2); }
template <class T>
inline T QuadReadAcrossDiagonal(const T& v) { return quad_read(v, 3); }

// Runs `entry` for every thread of groups.x * groups.y * groups.z groups of
// size gs. Groups are independent (the passes write disjoint pixels) and run in
// parallel unless `sequential`; with `lockstep` the threads of a group run as
// fibers (quad operations).
inline ThreadIds thread_ids(uint3 gs, uint3 g, uint32_t lx, uint32_t ly, uint32_t lz) {
  ThreadIds t;
  t.group_id = g;
  t.group_thread_id = uint3(lx, ly, lz);
  t.dispatch_thread_id = uint3(g.e[0] * gs.e[0] + lx, g.e[1] * gs.e[1] + ly, g.e[2] * gs.e[2] + lz);
  t.group_index = (lz * gs.e[1] + ly) * gs.e[0] + lx;
  return t;
}
inline void run_group_plain(void (*entry)(const ThreadIds&), uint3 gs, uint3 g) {
  for (uint32_t lz = 0; lz < gs.e[2]; ++lz)
    for (uint32_t ly = 0; ly < gs.e[1]; ++ly)
      for (uint32_t lx = 0; lx < gs.e[0]; ++lx) entry(thread_ids(gs, g, lx, ly, lz));
}
inline void run_group_fibers(void (*entry)(const ThreadIds&), uint3 gs, uint3 g, FiberGroup& fg) {
  const int n = (int)(gs.e[0] * gs.e[1] * gs.e[2]);
  fg.entry = entry;
  fg.fibers.resize(n);
  fg.quads.assign((n + 3) / 4, FiberGroup::QuadSlot());
  for (int i = 0; i < n; ++i) {
    Fiber& f = fg.fibers[i];
    const uint32_t lx = i % gs.e[0], ly = (i / gs.e[0]) % gs.e[1], lz = i / (gs.e[0] * gs.e[1]);
    f.ids = thread_ids(gs, g, lx, ly, lz);
    f.lane = (int)f.ids.group_index;
    f.done = false;
    f.group = &fg;
    if (f.stack.empty()) f.stack.resize(256 * 1024);
    getcontext(&f.ctx);
    f.ctx.uc_stack.ss_sp = f.stack.data();
    f.ctx.uc_stack.ss_size = f.stack.size();
    f.ctx.uc_link = nullptr;
    const uintptr_t pf = (uintptr_t)&f;
    makecontext(&f.ctx, (void (*)())fiber_trampoline, 2, (unsigned)(pf & 0xFFFFFFFFu), (unsigned)(pf >> 32));
  }
  cur_group() = &fg;
  for (bool any_left = true; any_left;) {
    any_left = false;
    for (int i = 0; i < n; ++i) {
      if (fg.fibers[i].done) continue;
      fg.current = i;
      swapcontext(&fg.sched, &fg.fibers[i].ctx);
      any_left = any_left || !fg.fibers[i].done;
    }
  }
  cur_group() = nullptr;
}

// Runs `entry` for every thread of groups.x * groups.y * groups.z groups of size gs.
// Groups run in parallel (OpenMP) unless `sequential` (passes with atomics run in
// dispatch order, which defines their result); with `lockstep` the threads of a
// group run as fibers (quad operations).
inline void dispatch(void (*entry)(const ThreadIds&), uint3 gs, uint3 groups, bool sequential, bool lockstep) {
  const long ng = (long)groups.e[0] * groups.e[1] * groups.e[2];
  auto group_of = [&](long k) {
    return uint3((uint32_t)(k % groups.e[0]), (uint32_t)((k / groups.e[0]) % groups.e[1]),
                 (uint32_t)(k / ((long)groups.e[0] * groups.e[1])));
  };
  if (sequential) {
    FiberGroup fg;
    for (long k = 0; k < ng; ++k) {
      if (lockstep) run_group_fibers(entry, gs, group_of(k), fg);
      else run_group_plain(entry, gs, group_of(k));
    }
    return;
  }
#pragma omp parallel
  {
    FiberGroup fg;
#pragma omp for schedule(dynamic, 16)
    for (long k = 0; k < ng; ++k) {
      if (lockstep) run_group_fibers(entry, gs, group_of(k), fg);
      else run_group_plain(entry, gs, group_of(k));
    }
  }
}

}  // namespace hlsl
