// device_common.cuh -- element types, vector loads/stores and the Kubelka-Munk math.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pg {

// ------------------------------------------------------------------ element conversion
__device__ __forceinline__ float to_f(float x) { return x; }
__device__ __forceinline__ float to_f(__half x) { return __half2float(x); }
__device__ __forceinline__ float to_f(__nv_bfloat16 x) { return __bfloat162float(x); }
__device__ __forceinline__ double to_d(double x) { return x; }

template <class T>
__device__ __forceinline__ T from_f(float x);
template <>
__device__ __forceinline__ float from_f<float>(float x) { return x; }
template <>
__device__ __forceinline__ __half from_f<__half>(float x) { return __float2half_rn(x); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float x) {
  return __float2bfloat16_rn(x);
}

// Math type for a storage type: double for double storage, float otherwise.
template <class T> struct MathOf { using type = float; };
template <> struct MathOf<double> { using type = double; };

template <class M, class T>
__device__ __forceinline__ M ld_elem(const T* p) { return static_cast<M>(to_f(*p)); }
template <>
__device__ __forceinline__ double ld_elem<double, double>(const double* p) { return *p; }
// L2 loads (bypassing L1): data other SMs of a cluster wrote before a cluster barrier.
template <class M, class T>
__device__ __forceinline__ M ld_cg(const T* p) { return static_cast<M>(to_f(__ldcg(p))); }
template <>
__device__ __forceinline__ double ld_cg<double, double>(const double* p) { return __ldcg(p); }
// Load through L1 (CG false) or from L2 only (CG true).
template <bool CG, class M, class T>
__device__ __forceinline__ M ld_sel(const T* p) {
  if constexpr (CG) return ld_cg<M>(p);
  else return ld_elem<M>(p);
}
template <class M, class T>
__device__ __forceinline__ void st_elem(T* p, M v) { *p = from_f<T>(static_cast<float>(v)); }
template <>
__device__ __forceinline__ void st_elem<double, double>(double* p, double v) { *p = v; }

// Stochastic rounding to a 16-bit storage type: `r` supplies the random low bits (13 for FP16,
// 16 for BF16), added to the FP32 pattern before truncation, so the stored value is
// unbiased. FP16 subnormals (|x| < 2^-14) round to nearest. FP32 / FP64 store exactly.
template <class T>
__device__ __forceinline__ T from_f_sr(float x, uint32_t r);
template <>
__device__ __forceinline__ float from_f_sr<float>(float x, uint32_t) { return x; }
template <>
__device__ __forceinline__ __half from_f_sr<__half>(float x, uint32_t r) {
  if (!(fabsf(x) >= 6.103515625e-05f) || !(fabsf(x) < 65504.0f)) return __float2half_rn(x);
  return __float2half_rz(__uint_as_float(__float_as_uint(x) + (r & 0x1fffu)));
}
template <>
__device__ __forceinline__ __nv_bfloat16 from_f_sr<__nv_bfloat16>(float x, uint32_t r) {
  if (!(fabsf(x) < 3.0e38f)) return __float2bfloat16_rn(x);
  return __float2bfloat16_rz(__uint_as_float(__float_as_uint(x) + (r & 0xffffu)));
}
// The storage value of v (stochastically rounded for 16-bit types).
template <class T, class M>
__device__ __forceinline__ T to_store_sr(M v, uint32_t r) {
  return from_f_sr<T>(static_cast<float>(v), r);
}
template <>
__device__ __forceinline__ double to_store_sr<double, double>(double v, uint32_t) {
  return v;
}
template <class M, class T>
__device__ __forceinline__ void st_elem_sr(T* p, M v, uint32_t r) {
  *p = to_store_sr<T>(v, r);
}

// ------------------------------------------------------------------ bounds-checked builds
// A library built with PAINTY_BOUNDS_CHECK (libpainty_gb300_checked.so) tests the computed
// indices of the stamp kernels against their buffers' extents before each access. An index
// outside is recorded -- bit kStatusBounds in status word 0, the first such access's kind in
// word 4 and its index in word 5 -- and the access is skipped instead of faulting. The host
// turns a recorded access into an error naming them.
#ifdef PAINTY_BOUNDS_CHECK
constexpr bool kBoundsCheck = true;
#else
constexpr bool kBoundsCheck = false;
#endif
constexpr unsigned kStatusBounds = 4u;
enum BoundsKind : unsigned {
  kBoundsCanvas = 1,    // canvas / snapshot pixel record
  kBoundsCell = 2,      // pickup-map cell
  kBoundsFootprint = 3, // footprint height
  kBoundsCellMap = 4,   // per-stamp cell map
  kBoundsOwner = 5,     // owner table
  kBoundsDescriptor = 6,  // batch descriptors (canvas, stroke, path points, footprint, slot)
};
__device__ __forceinline__ bool in_bounds(unsigned* status, unsigned kind, int64_t idx,
                                          int64_t n) {
  if constexpr (!kBoundsCheck) {
    return true;
  } else {
    if (idx >= 0 && idx < n) return true;
    if (status) {
      atomicOr(status, kStatusBounds);
      if (atomicCAS(status + 4, 0u, kind) == 0u) atomicExch(status + 5, static_cast<unsigned>(idx));
    }
    return false;
  }
}

// ------------------------------------------------------------------ thread-block clusters
// Rank of this CTA in its cluster and the cluster's size (1 and 0 without a cluster launch).
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
// Barrier over every thread of the cluster; memory operations before it (global and shared,
// by any CTA of the cluster) are visible after it. All threads call it, convergently.
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;"
               ::: "memory");
}

// The record of one pixel of a packed layer: 8 elements of the storage size (K r,g,b, S r,g,b,
// V, pad) read and written as 16-byte words.
template <class TK, class TV>
union PixRec {
  static constexpr int kWords = 8 * sizeof(TK) / 16;
  uint4 w[kWords];
  TK k[8];
  TV v[8];
};
template <bool CG, class TK, class TV>
__device__ __forceinline__ PixRec<TK, TV> load_rec(const void* base, int c) {
  using R = PixRec<TK, TV>;
  const uint4* p = static_cast<const uint4*>(base) + static_cast<int64_t>(c) * R::kWords;
  R r;
#pragma unroll
  for (int i = 0; i < R::kWords; i++) {
    if constexpr (CG) r.w[i] = __ldcg(p + i);
    else r.w[i] = p[i];
  }
  return r;
}
template <class TK, class TV>
__device__ __forceinline__ void store_rec(void* base, int c, const PixRec<TK, TV>& r) {
  using R = PixRec<TK, TV>;
  uint4* p = static_cast<uint4*>(base) + static_cast<int64_t>(c) * R::kWords;
#pragma unroll
  for (int i = 0; i < R::kWords; i++) p[i] = r.w[i];
}
template <class TK, class TV>
__device__ __forceinline__ TV* rec_v(void* base, int c) {
  return reinterpret_cast<TV*>(static_cast<char*>(base) + static_cast<int64_t>(c) * 8 * sizeof(TK)) + 6;
}

// 32-bit integer hash (xorshift-multiply finaliser) for the rounding bits.
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// ------------------------------------------------------------------ streaming 16-byte I/O
// Streaming (read-once) 128-bit loads that do not allocate in L1, and streaming stores.
__device__ __forceinline__ uint4 ld_stream_u4(const void* p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}
__device__ __forceinline__ uint2 ld_stream_u2(const void* p) {
  uint2 r;
  asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0,%1}, [%2];"
               : "=r"(r.x), "=r"(r.y)
               : "l"(p));
  return r;
}
__device__ __forceinline__ void st_stream_u4(void* p, uint4 v) {
  asm volatile("st.global.cs.v4.u32 [%0], {%1,%2,%3,%4};" ::"l"(p), "r"(v.x), "r"(v.y),
               "r"(v.z), "r"(v.w)
               : "memory");
}

// ------------------------------------------------------------------ N-element vector I/O
// N elements of T as 16-byte streaming loads / stores (N * sizeof(T) a multiple of 16).
template <int N, class T>
__device__ __forceinline__ void load_vec(const T* p, T (&o)[N]) {
  static_assert((N * sizeof(T)) % 16 == 0, "whole 16-byte vectors");
  constexpr int V = N * sizeof(T) / 16;
  uint4 raw[V];
#pragma unroll
  for (int v = 0; v < V; v++) raw[v] = ld_stream_u4(reinterpret_cast<const char*>(p) + 16 * v);
  const T* e = reinterpret_cast<const T*>(raw);
#pragma unroll
  for (int i = 0; i < N; i++) o[i] = e[i];
}
template <int N, class T>
__device__ __forceinline__ void store_vec(T* p, const T (&v)[N]) {
  static_assert((N * sizeof(T)) % 16 == 0, "whole 16-byte vectors");
  constexpr int V = N * sizeof(T) / 16;
  uint4 raw[V];
  T* e = reinterpret_cast<T*>(raw);
#pragma unroll
  for (int i = 0; i < N; i++) e[i] = v[i];
#pragma unroll
  for (int w = 0; w < V; w++) st_stream_u4(reinterpret_cast<char*>(p) + 16 * w, raw[w]);
}

// ------------------------------------------------------------------ hardware approximations
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// ------------------------------------------------------------------ Kubelka-Munk
// Reflectance of a layer (K, S, thickness d) over a substrate of reflectance R0, with the
// semantics of painty's ComputeReflectance (painty/core/KubelkaMunk.hxx:25-83): R0 when
// |d| < 1e4*DBL_EPSILON, S replaced by 1e-11 when |S| <= 1e4*DBL_EPSILON.
//
// FP32 evaluation, rearranged to avoid cancellation and to need 3 MUFU operations:
//   with b = sqrt(a^2 - 1), a = 1 + K/S, x = b S d, and beta = S b = sqrt(K (2S + K)),
//   A = S (1 - R0) - R0 K, B = S (1 - R0) + K, e = exp(-2x):
//     R = (A u + R0 w) / (B u + w),   (u, w) = (1 - e, beta (1 + e))
//   and for x < 0.05, with g = x coth x = 1 + x^2/3 - x^4/45 (+ O(x^6) < 4e-11):
//     (u, w) = (d, g)
// Both are the reference's (1 - R0 (a - b coth x)) / (a - R0 + b coth x) multiplied through
// by S (1 - e) or by S d / g. The series form is finite at K = 0, where the reference's
// 0 * coth(0) is NaN. Branch-free: both forms are evaluated and selected. Physical inputs
// (K, S >= 0, d >= 0) are assumed.
__device__ __forceinline__ float km_reflectance(float K, float S, float R0, float d) {
  constexpr float kEps = 2.220446049250313e-12f;  // 1e4 * DBL_EPSILON
  S = fabsf(S) > kEps ? S : 1e-11f;
  const float q = fmaxf(K * (2.0f * S + K), 1e-30f);
  const float beta = q * rsqrt_approx(q);
  const float x = beta * d;
  const float omr = 1.0f - R0;
  const float A = fmaf(S, omr, -R0 * K);
  const float B = fmaf(S, omr, K);
  const float e = ex2_approx(-2.8853900817779268f * x);  // exp(-2x) = 2^(-2x log2 e)
  const float x2 = x * x;
  const float g = fmaf(x2, fmaf(x2, -1.0f / 45.0f, 1.0f / 3.0f), 1.0f);
  const bool series = x < 0.05f;
  const float u = series ? d : 1.0f - e;
  const float w = series ? g : beta * (1.0f + e);
  const float r = fmaf(A, u, R0 * w) * rcp_approx(fmaf(B, u, w));
  return fabsf(d) < kEps ? R0 : r;
}

// km_reflectance for two pixels at once on Blackwell's packed FP32 pipe (FFMA2 / FMUL2 /
// FADD2 each do two lanes of the scalar operation with the same rounding): the same formula,
// with every multiply-add written as an explicit fma, in about half the issued instructions.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 km_reflectance2(float2 K, float2 S, float2 R0, float2 d) {
  constexpr float kEps = 2.220446049250313e-12f;  // 1e4 * DBL_EPSILON
  S.x = fabsf(S.x) > kEps ? S.x : 1e-11f;
  S.y = fabsf(S.y) > kEps ? S.y : 1e-11f;
  const float2 one = f2(1.0f, 1.0f);
  float2 q = __fmul2_rn(K, __ffma2_rn(f2(2.0f, 2.0f), S, K));  // K (2S + K)
  q.x = fmaxf(q.x, 1e-30f);
  q.y = fmaxf(q.y, 1e-30f);
  const float2 beta = __fmul2_rn(q, f2(rsqrt_approx(q.x), rsqrt_approx(q.y)));
  const float2 x = __fmul2_rn(beta, d);
  const float2 nR0 = f2(-R0.x, -R0.y);
  const float2 omr = __fadd2_rn(one, nR0);
  const float2 A = __ffma2_rn(S, omr, __fmul2_rn(nR0, K));
  const float2 B = __ffma2_rn(S, omr, K);
  const float2 t = __fmul2_rn(f2(-2.8853900817779268f, -2.8853900817779268f), x);
  const float2 e = f2(ex2_approx(t.x), ex2_approx(t.y));  // exp(-2x)
  const float2 x2 = __fmul2_rn(x, x);
  const float2 g = __ffma2_rn(x2, __ffma2_rn(x2, f2(-1.0f / 45.0f, -1.0f / 45.0f),
                                              f2(1.0f / 3.0f, 1.0f / 3.0f)), one);
  const float2 ome = __fadd2_rn(one, f2(-e.x, -e.y));
  const float2 bope = __fmul2_rn(beta, __fadd2_rn(one, e));
  const bool sx = x.x < 0.05f, sy = x.y < 0.05f;
  const float2 u = f2(sx ? d.x : ome.x, sy ? d.y : ome.y);
  const float2 w = f2(sx ? g.x : bope.x, sy ? g.y : bope.y);
  const float2 num = __ffma2_rn(A, u, __fmul2_rn(R0, w));
  const float2 den = __ffma2_rn(B, u, w);
  const float2 r = __fmul2_rn(num, f2(rcp_approx(den.x), rcp_approx(den.y)));
  return f2(fabsf(d.x) < kEps ? R0.x : r.x, fabsf(d.y) < kEps ? R0.y : r.y);
}

// The three colour channels of two pixels, with one reciprocal per pixel instead of one per
// channel: R_c = N_c / D_c = N_c * (product of the other two D) / (D_r D_g D_b). D lies
// between about 0.03 and 30, so the product stays far inside FP32's range; the extra products
// cost a few roundings (well below FP16 storage's).
// kGuards: painty's two guards -- S replaced by 1e-11 where |S| <= 1e4 DBL_EPSILON (it
// divides by S), and R kept where |d| < 1e4 DBL_EPSILON. 16-bit layers skip both. This form
// never divides by S, so the substitution moves R by about 1e-11 relative, below FP32's
// resolution. Thickness stored as FP16 is either 0 or at least 2^-24, and at d = +-0 the
// formula itself returns R exactly (x = 0 takes the series: u = d = 0, w = g = 1, so every
// numerator is R, every denominator 1 and the reciprocal of their product 1).
template <bool kGuards = true>
__device__ __forceinline__ void km_reflectance2x3(const float2 (&K)[3], const float2 (&S)[3],
                                                  float2 (&R)[3], float2 d) {
  constexpr float kEps = 2.220446049250313e-12f;  // 1e4 * DBL_EPSILON
  const float2 one = f2(1.0f, 1.0f);
  float2 num[3], den[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    float2 s = S[c];
    if constexpr (kGuards) {
      s.x = fabsf(s.x) > kEps ? s.x : 1e-11f;
      s.y = fabsf(s.y) > kEps ? s.y : 1e-11f;
    }
    float2 q = __fmul2_rn(K[c], __ffma2_rn(f2(2.0f, 2.0f), s, K[c]));
    q.x = fmaxf(q.x, 1e-30f);
    q.y = fmaxf(q.y, 1e-30f);
    const float2 beta = __fmul2_rn(q, f2(rsqrt_approx(q.x), rsqrt_approx(q.y)));
    const float2 x = __fmul2_rn(beta, d);
    const float2 nR0 = f2(-R[c].x, -R[c].y);
    const float2 omr = __fadd2_rn(one, nR0);
    const float2 A = __ffma2_rn(s, omr, __fmul2_rn(nR0, K[c]));
    const float2 B = __ffma2_rn(s, omr, K[c]);
    const float2 t = __fmul2_rn(f2(-2.8853900817779268f, -2.8853900817779268f), x);
    const float2 e = f2(ex2_approx(t.x), ex2_approx(t.y));  // exp(-2x)
    const float2 x2 = __fmul2_rn(x, x);
    const float2 g = __ffma2_rn(x2, __ffma2_rn(x2, f2(-1.0f / 45.0f, -1.0f / 45.0f),
                                                f2(1.0f / 3.0f, 1.0f / 3.0f)), one);
    const float2 ome = __fadd2_rn(one, f2(-e.x, -e.y));
    const float2 bope = __fmul2_rn(beta, __fadd2_rn(one, e));
    const bool sx = x.x < 0.05f, sy = x.y < 0.05f;
    const float2 u = f2(sx ? d.x : ome.x, sy ? d.y : ome.y);
    const float2 w = f2(sx ? g.x : bope.x, sy ? g.y : bope.y);
    num[c] = __ffma2_rn(A, u, __fmul2_rn(R[c], w));
    den[c] = __ffma2_rn(B, u, w);
  }
  const float2 d01 = __fmul2_rn(den[0], den[1]);
  const float2 d12 = __fmul2_rn(den[1], den[2]);
  const float2 d02 = __fmul2_rn(den[0], den[2]);
  const float2 all = __fmul2_rn(d01, den[2]);
  const float2 inv = f2(rcp_approx(all.x), rcp_approx(all.y));
  const float2 o[3] = {__fmul2_rn(__fmul2_rn(num[0], d12), inv),
                       __fmul2_rn(__fmul2_rn(num[1], d02), inv),
                       __fmul2_rn(__fmul2_rn(num[2], d01), inv)};
  if constexpr (kGuards) {
    const bool keep_x = fabsf(d.x) < kEps, keep_y = fabsf(d.y) < kEps;
#pragma unroll
    for (int c = 0; c < 3; c++) R[c] = f2(keep_x ? R[c].x : o[c].x, keep_y ? R[c].y : o[c].y);
  } else {
#pragma unroll
    for (int c = 0; c < 3; c++) R[c] = o[c];
  }
}

// painty's coth (painty/core/Math.hxx:157-169) and ComputeReflectance in double, in the
// reference's own operation order; for the F64 parity storage mode.
__device__ __forceinline__ double coth_ref(double x) {
  if (x > 20.0) return 1.0;
  if (fabs(x) > 0.0) {
    const double res = cosh(x) / sinh(x);
    return isnan(res) ? 1.0 : res;
  }
  return __longlong_as_double(0x7ff0000000000000ULL);
}
__device__ __forceinline__ double km_reflectance(double K, double S_in, double R0, double d) {
  constexpr double kEps = 2.220446049250313e-12;
  if (fabs(d) < kEps) return R0;
  const double S = fabs(S_in) > kEps ? S_in : 0.00000000001;
  const double K_S = __ddiv_rn(K, S);
  const double a = __dadd_rn(1.0, K_S);
  const double v = __dadd_rn(__dmul_rn(a, a), -1.0);
  const double b = v < 0.0 ? 0.0 : __dsqrt_rn(v);
  const double bSh = __dmul_rn(__dmul_rn(b, S), d);
  const double bc = __dmul_rn(b, coth_ref(bSh));
  return __ddiv_rn(__dadd_rn(1.0, -__dmul_rn(R0, __dadd_rn(a, -bc))),
                   __dadd_rn(__dadd_rn(a, -R0), bc));
}

}  // namespace pg
