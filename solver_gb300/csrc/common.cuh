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
