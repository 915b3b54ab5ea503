// Shared device/host helpers for the GB300 FFT-PEEC kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>

template <typename R>
struct alignas(2 * sizeof(R)) cx {
  R x, y;
};
using c64 = cx<double>;
using c32 = cx<float>;

template <typename R>
__host__ __device__ __forceinline__ cx<R> mk(R a, R b) {
  cx<R> r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) {
  return mk<R>(a.x + b.x, a.y + b.y);
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) {
  return mk<R>(a.x - b.x, a.y - b.y);
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
  return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> cmulc(cx<R> a, cx<R> b) {  // a * conj(b)
  return mk<R>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> cscale(cx<R> a, R s) {
  return mk<R>(a.x * s, a.y * s);
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> cconj(cx<R> a) {
  return mk<R>(a.x, -a.y);
}
template <typename To, typename From>
__host__ __device__ __forceinline__ cx<To> ccast(cx<From> a) {
  return mk<To>((To)a.x, (To)a.y);
}

__host__ __device__ __forceinline__ int ilog2(int v) {
  int r = 0;
  while ((1 << r) < v) ++r;
  return r;
}
__host__ __device__ __forceinline__ int brev(int v, int bits) {
  int r = 0;
  for (int i = 0; i < bits; ++i) {
    r = (r << 1) | (v & 1);
    v >>= 1;
  }
  return r;
}

#define PEEC_CUDA_TRY(expr)                                       \
  do {                                                            \
    cudaError_t _e = (expr);                                      \
    if (_e != cudaSuccess) return peec::fail_cuda(_e, #expr, __FILE__, __LINE__); \
  } while (0)

// Float-float ("double-float") scalar: value = hi + lo with |lo| <= ulp(hi)/2, about 48
// significant bits from FP32 arithmetic. Error-free transformations (Knuth two-sum,
// Dekker fast two-sum, FMA two-product) use the _rn intrinsics so the compiler can
// neither contract nor reassociate them. Used for the refinement residual operator,
// where GB300's FP32 pipes are far faster than its FP64 ones.
struct ff {
  float hi, lo;
  ff() = default;
  __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ ff(int i) : ff((double)i) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

#ifdef __CUDA_ARCH__
#define PEEC_FADD(a, b) __fadd_rn(a, b)
#define PEEC_FSUB(a, b) __fsub_rn(a, b)
#define PEEC_FMUL(a, b) __fmul_rn(a, b)
#define PEEC_FMA(a, b, c) __fmaf_rn(a, b, c)
#else
#define PEEC_FADD(a, b) ((a) + (b))
#define PEEC_FSUB(a, b) ((a) - (b))
#define PEEC_FMUL(a, b) ((a) * (b))
#define PEEC_FMA(a, b, c) fmaf(a, b, c)
#endif

__host__ __device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = PEEC_FADD(a, b);
  const float bb = PEEC_FSUB(s, a);
  const float e = PEEC_FADD(PEEC_FSUB(a, PEEC_FSUB(s, bb)), PEEC_FSUB(b, bb));
  return ff(s, e);
}
__host__ __device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = PEEC_FADD(a, b);
  return ff(s, PEEC_FSUB(b, PEEC_FSUB(s, a)));
}
// Sum with the low parts added in FP32 after an exact two-sum of the high parts: the
// error is within a few units of 2^-48 (|a| + |b|), which is the norm-wise accuracy
// the transforms need (their error bounds are norm-wise, not element-wise).
__host__ __device__ __forceinline__ ff operator+(ff a, ff b) {
  const ff s = ff_two_sum(a.hi, b.hi);
  return ff_fast_two_sum(s.hi, PEEC_FADD(s.lo, PEEC_FADD(a.lo, b.lo)));
}
__host__ __device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__host__ __device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = PEEC_FMUL(a.hi, b.hi);
  float e = PEEC_FMA(a.hi, b.hi, -p);
  e = PEEC_FMA(a.hi, b.lo, e);
  e = PEEC_FMA(a.lo, b.hi, e);
  return ff_fast_two_sum(p, e);
}
using cff = cx<ff>;
