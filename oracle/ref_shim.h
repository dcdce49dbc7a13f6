// ORACLE -- test infrastructure only.
//
// OpenCL C shim that lets the reference's own Kernels.cl compile as C++ for the CPU
// (oracle/build_ref.py).  It provides the OpenCL vector types used by the kernels
// (float2/4/8, int2/4, uchar2/4, uint4) with the swizzle members the file uses, the
// arithmetic on them, the conversion/reinterpretation built-ins, and work-item ids.
//
// Implementation choices where OpenCL leaves room, identical to the restatement in
// oracle/raster_oracle.cpp: IEEE single precision with no contraction; min/max are
// selects (OpenCL's definition); fmin/fmax return the other argument for a NaN;
// convert_int rounds toward zero and saturates (NaN -> 0); convert_uchar rounds
// toward zero and clamps to [0,255] (NaN -> 0).
#ifndef GUDNI_REF_SHIM_H
#define GUDNI_REF_SHIM_H

#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

using std::isinf;

typedef unsigned int uint;
typedef unsigned long ulong;
typedef unsigned char uchar;
typedef unsigned short ushort;

#pragma GCC diagnostic ignored "-Wpedantic"
#pragma GCC diagnostic ignored "-Wunused-function"
#pragma GCC diagnostic ignored "-Wunused-variable"
#pragma GCC diagnostic ignored "-Wunused-parameter"

struct alignas(8) float2 { union { struct { float x, y; }; struct { float s0, s1; }; }; };
struct alignas(16) float4 {
  union {
    struct { float x, y, z, w; };
    struct { float s0, s1, s2, s3; };
    struct { float2 xy, zw; };
  };
};
struct alignas(32) float8 {
  union {
    struct { float s0, s1, s2, s3, s4, s5, s6, s7; };
    struct { float4 s0123, s4567; };
  };
};
struct alignas(8) int2 { union { struct { int x, y; }; struct { int s0, s1; }; }; };
struct alignas(16) int4 {
  union {
    struct { int x, y, z, w; };
    struct { int2 xy, zw; };
  };
};
struct alignas(16) uint4 { union { struct { uint x, y, z, w; }; struct { uint s0, s1, s2, s3; }; }; };
struct alignas(2) uchar2 { union { struct { uchar x, y; }; struct { uchar s0, s1; }; }; };
struct alignas(4) uchar4 {
  union {
    struct { uchar x, y, z, w; };
    struct { uchar s0, s1, s2, s3; };
    struct { uchar2 xy, zw; };
  };
};

template <class V> struct ocl_traits;
template <> struct ocl_traits<float2> { using T = float; static constexpr int N = 2; };
template <> struct ocl_traits<float4> { using T = float; static constexpr int N = 4; };
template <> struct ocl_traits<float8> { using T = float; static constexpr int N = 8; };
template <> struct ocl_traits<int2> { using T = int; static constexpr int N = 2; };
template <> struct ocl_traits<int4> { using T = int; static constexpr int N = 4; };
template <> struct ocl_traits<uint4> { using T = uint; static constexpr int N = 4; };
template <> struct ocl_traits<uchar2> { using T = uchar; static constexpr int N = 2; };
template <> struct ocl_traits<uchar4> { using T = uchar; static constexpr int N = 4; };

template <class V> inline typename ocl_traits<V>::T* ocl_lanes(V& v) {
  return reinterpret_cast<typename ocl_traits<V>::T*>(&v);
}
template <class V> inline const typename ocl_traits<V>::T* ocl_lanes(const V& v) {
  return reinterpret_cast<const typename ocl_traits<V>::T*>(&v);
}

template <class T, class = void> struct ocl_is_vec : std::false_type {};
template <class T> struct ocl_is_vec<T, std::void_t<decltype(ocl_traits<T>::N)>> : std::true_type {};

// Vector literal (V)(a, b, ...): components are concatenated; one scalar broadcasts.
template <class V, class E>
inline void ocl_fill(V& v, int& k, const E& e) {
  using T = typename ocl_traits<V>::T;
  if constexpr (ocl_is_vec<E>::value) {
    for (int i = 0; i < ocl_traits<E>::N; ++i) ocl_lanes(v)[k++] = (T)ocl_lanes(e)[i];
  } else {
    ocl_lanes(v)[k++] = (T)e;
  }
}
template <class V, class... A>
inline V ocl_make(const A&... a) {
  V v;
  std::memset(&v, 0, sizeof(V));
  int k = 0;
  (ocl_fill(v, k, a), ...);
  if (k == 1) {
    for (int i = 1; i < ocl_traits<V>::N; ++i) ocl_lanes(v)[i] = ocl_lanes(v)[0];
  }
  return v;
}

#define OCL_BINOP(OP)                                                                         \
  template <class V, class = std::enable_if_t<ocl_is_vec<V>::value>>                           \
  inline V operator OP(const V& a, const V& b) {                                               \
    V r;                                                                                       \
    for (int i = 0; i < ocl_traits<V>::N; ++i) ocl_lanes(r)[i] = ocl_lanes(a)[i] OP ocl_lanes(b)[i]; \
    return r;                                                                                  \
  }                                                                                            \
  template <class V, class S, class = std::enable_if_t<ocl_is_vec<V>::value && std::is_arithmetic<S>::value>> \
  inline V operator OP(const V& a, S s) {                                                      \
    V r;                                                                                       \
    using T = typename ocl_traits<V>::T;                                                       \
    for (int i = 0; i < ocl_traits<V>::N; ++i) ocl_lanes(r)[i] = ocl_lanes(a)[i] OP (T)s;     \
    return r;                                                                                  \
  }                                                                                            \
  template <class V, class S, class = std::enable_if_t<ocl_is_vec<V>::value && std::is_arithmetic<S>::value>> \
  inline V operator OP(S s, const V& a) {                                                      \
    V r;                                                                                       \
    using T = typename ocl_traits<V>::T;                                                       \
    for (int i = 0; i < ocl_traits<V>::N; ++i) ocl_lanes(r)[i] = (T)s OP ocl_lanes(a)[i];     \
    return r;                                                                                  \
  }                                                                                            \
  template <class V, class = std::enable_if_t<ocl_is_vec<V>::value>>                           \
  inline V& operator OP##=(V& a, const V& b) {                                                 \
    a = a OP b;                                                                                \
    return a;                                                                                  \
  }

OCL_BINOP(+)
OCL_BINOP(-)
OCL_BINOP(*)
OCL_BINOP(/)

// min / max (OpenCL common functions): y if y < x (min) / x < y (max), else x.
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline int min(int x, int y) { return y < x ? y : x; }
inline int max(int x, int y) { return x < y ? y : x; }
inline float fmin(float x, float y) { return std::isnan(y) ? x : (std::isnan(x) ? y : min(x, y)); }
inline float fmax(float x, float y) { return std::isnan(y) ? x : (std::isnan(x) ? y : max(x, y)); }
inline float fabs(float x) { return std::fabs(x); }

inline ulong clz(ulong v) { return v == 0 ? 64ul : (ulong)__builtin_clzl(v); }
inline int mul24(int a, int b) { return a * b; }

inline int ocl_to_int_rtz(float v) {
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0f) return 2147483647;
  if (v <= -2147483648.0f) return (-2147483647 - 1);
  return (int)v;
}
inline uchar ocl_to_uchar_rtz(float v) {
  if (!(v > 0.0f)) return 0;
  if (v >= 255.0f) return 255;
  return (uchar)(int)v;
}
inline int2 convert_int2(float2 v) { return ocl_make<int2>(ocl_to_int_rtz(v.x), ocl_to_int_rtz(v.y)); }
inline float2 convert_float2(int2 v) { return ocl_make<float2>((float)v.x, (float)v.y); }
inline float convert_float(int v) { return (float)v; }
inline float4 convert_float4(uchar4 v) {
  return ocl_make<float4>((float)v.s0, (float)v.s1, (float)v.s2, (float)v.s3);
}
inline uchar4 convert_uchar4(float4 v) {
  return ocl_make<uchar4>(ocl_to_uchar_rtz(v.s0), ocl_to_uchar_rtz(v.s1), ocl_to_uchar_rtz(v.s2),
                          ocl_to_uchar_rtz(v.s3));
}

template <class To, class From>
inline To ocl_bits(const From& f) {
  static_assert(sizeof(To) == sizeof(From), "as_* needs equal sizes");
  To t;
  std::memcpy(&t, &f, sizeof(To));
  return t;
}
inline uint as_uint(float f) { return ocl_bits<uint>(f); }
inline uint as_uint(uchar4 v) { return ocl_bits<uint>(v); }
inline uint4 as_uint4(float4 v) { return ocl_bits<uint4>(v); }
inline ushort as_ushort(uchar2 v) { return ocl_bits<ushort>(v); }
inline uchar4 as_uchar4(uint v) { return ocl_bits<uchar4>(v); }
inline float as_float(uint v) { return ocl_bits<float>(v); }

// work-item ids, set by the driver loop before each kernel call
extern thread_local size_t gudni_ref_gid[2];
inline size_t get_global_id(int d) { return gudni_ref_gid[d]; }

// MAXTHRESHOLDS is a runtime capacity here (it only sizes the per-column slabs)
extern int gudni_ref_max_thresholds;

#define __kernel
#define __global
#define __local
#define __constant
#define __private
#define printf(...) ((void)0)
// Kernels.cl:813 declares pos2 with an old-style (K&R) parameter list
#define pos2(x, y, width) gudni_ref_pos2_(int x, int y, int width)
// C++ keyword used as a parameter name in Kernels.cl
#define new new_

#endif  // GUDNI_REF_SHIM_H
