// Dense operator products of the RIS solver (compute_matrix_vector.jl:14-25): the three
// partial-inductance blocks Lp_x, Lp_y, Lp_z times the edge currents and the dense
// potential matrix P times the surface charges, for real column-major n x n blocks
// (the reference's Lp_data / P_data) and complex vectors.
//
// The work is a matrix-vector product that reads every matrix entry once: 8 bytes (FP64
// storage) or 4 bytes (FP32 storage, the inner solves of the mixed solve) for four flops
// (the real and imaginary parts). In FP64 that is bound by GB300's FP64 rate (about 1/60 of
// FP32); the FP32 copy runs at HBM speed. Layout: a CTA owns 256 consecutive rows and one
// chunk of columns; a warp reads 32 consecutive rows of one column per step (128 or 256
// contiguous bytes), the chunk's vector entries sit in shared memory, and eight columns
// are in flight per thread. Each chunk writes its partial sums; a second kernel adds them
// in chunk order, so results do not depend on scheduling.
#include "ctx.hpp"

namespace peec {

constexpr int DN_TPB = 256;
constexpr int DN_CHUNK_MAX = 2048;  // columns per chunk (the vector slice in shared memory)

template <typename T>
__global__ void __launch_bounds__(DN_TPB) k_dense_gemv(const T* __restrict__ M, int64_t n,
                                                       const c64* __restrict__ x, int cols,
                                                       int offdiag, c64* __restrict__ part) {
  __shared__ cx<T> xs[DN_CHUNK_MAX];
  const int64_t c0 = (int64_t)blockIdx.y * cols;
  const int64_t c1 = min(c0 + cols, n);
  for (int64_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
    const c64 v = x[j];
    xs[j - c0] = mk<T>((T)v.x, (T)v.y);
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * DN_TPB + threadIdx.x;
  if (i >= n) return;
  T ar = 0, ai = 0;
  const T* __restrict__ col = M + c0 * n + i;
  int64_t j = c0;
  for (; j + 8 <= c1; j += 8) {
    T mv[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mv[q] = col[(size_t)q * n];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const T m = (offdiag && j + q == i) ? T(0) : mv[q];
      const cx<T> xv = xs[j + q - c0];
      ar = ar + m * xv.x;
      ai = ai + m * xv.y;
    }
    col += (size_t)8 * n;
  }
  for (; j < c1; ++j, col += n) {
    const T m = (offdiag && j == i) ? T(0) : *col;
    const cx<T> xv = xs[j - c0];
    ar = ar + m * xv.x;
    ai = ai + m * xv.y;
  }
  part[(size_t)blockIdx.y * n + i] = mk<double>((double)ar, (double)ai);
}

// out[i] = sum over chunks of part[chunk][i], chunks in order
__global__ void k_dense_sum(const c64* __restrict__ part, int nchunk, int64_t n, c64* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    c64 s = part[i];
    for (int c = 1; c < nchunk; ++c) s = s + part[(size_t)c * n + i];
    out[i] = s;
  }
}

// column chunks of an n x n product: enough CTAs for every SM (about 8 per SM), at most
// DN_CHUNK_MAX columns each
int dense_chunks(int64_t n) {
  if (n <= 0) return 1;
  const int64_t tiles = (n + DN_TPB - 1) / DN_TPB;
  int64_t c = (152 * 8 + tiles - 1) / tiles;
  const int64_t cmin = (n + DN_CHUNK_MAX - 1) / DN_CHUNK_MAX;
  const int64_t cmax = std::max<int64_t>(1, n / 64);
  if (c > cmax) c = cmax;
  if (c < cmin) c = cmin;
  return (int)c;
}

// out = M x (offdiag: without M's diagonal) for one real n x n block; part holds
// dense_chunks(n) * n entries. Returns the kernels launched.
int dense_apply(const void* M, bool fp32, int64_t n, const c64* x, int offdiag, c64* part,
                c64* out, cudaStream_t st) {
  if (n <= 0) return 0;
  const int nc = dense_chunks(n);
  const int cols = (int)((n + nc - 1) / nc);
  const dim3 grid((unsigned)((n + DN_TPB - 1) / DN_TPB), (unsigned)nc);
  if (fp32)
    k_dense_gemv<float><<<grid, DN_TPB, 0, st>>>((const float*)M, n, x, cols, offdiag, part);
  else
    k_dense_gemv<double><<<grid, DN_TPB, 0, st>>>((const double*)M, n, x, cols, offdiag, part);
  int64_t b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  k_dense_sum<<<(unsigned)b, 256, 0, st>>>(part, nc, n, out);
  return 2;
}

// FP32 copy of an FP64 array (the mixed solve's matrices), on the device
__global__ void k_dense_round(const double* __restrict__ a, size_t cnt, float* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < cnt;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)a[i];
}

void dense_round(const double* a, size_t cnt, float* out, cudaStream_t st) {
  size_t b = (cnt + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  k_dense_round<<<(unsigned)b, 256, 0, st>>>(a, cnt, out);
}

}  // namespace peec
