// Dense operator products of the RIS solver (compute_matrix_vector.jl:14-25): the three
// partial-inductance blocks Lp_x, Lp_y, Lp_z times the edge currents and the dense
// potential matrix P times the surface charges, for real column-major n x n blocks
// (the reference's Lp_data / P_data) and complex vectors.
//
// The work is a matrix-vector product that reads every matrix entry once: 8 bytes (FP64
// storage) or 4 bytes (FP32 storage, the inner solves of the mixed solve) for four flops
// (the real and imaginary parts). In FP64 that is bound by GB300's FP64 rate (about 1/60 of
// FP32); the FP32 copy runs at HBM speed. Layout: the matrices are stored column-major
// with the leading dimension padded to a multiple of 4; a thread owns 4 (FP32) or 2 (FP64)
// consecutive rows and reads them with one 16-byte load per column (a warp: 512 contiguous
// bytes); a CTA owns 256 threads' rows and one chunk of columns, whose vector entries sit
// in shared memory; eight columns are in flight per thread. Each chunk writes its partial
// sums; a second kernel adds them in chunk order, so results do not depend on scheduling.
#include <algorithm>
#include <atomic>

#include "ctx.hpp"

namespace peec {

constexpr int DN_TPB = 256;
constexpr int DN_CHUNK_MAX = 2048;  // columns per chunk (the vector slice in shared memory)

// rows per thread: one 16-byte load per column (4 floats or 2 doubles)
template <typename T> struct DnVec;
template <> struct DnVec<float> { using V = float4; static constexpr int R = 4; };
template <> struct DnVec<double> { using V = double2; static constexpr int R = 2; };
template <typename T, typename V>
__device__ __forceinline__ T dn_at(const V& v, int r) {
  return reinterpret_cast<const T*>(&v)[r];
}

// M: n x n, column-major with leading dimension ld (a multiple of 4, rows n..ld zero)
template <typename T>
__global__ void __launch_bounds__(DN_TPB) k_dense_gemv(const T* __restrict__ M, int64_t n,
                                                       int64_t ld, const c64* __restrict__ x,
                                                       int cols, int offdiag,
                                                       c64* __restrict__ part) {
  using V = typename DnVec<T>::V;
  constexpr int R = DnVec<T>::R;
  __shared__ cx<T> xs[DN_CHUNK_MAX];
  const int64_t c0 = (int64_t)blockIdx.y * cols;
  const int64_t c1 = min(c0 + cols, n);
  for (int64_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
    const c64 v = x[j];
    xs[j - c0] = mk<T>((T)v.x, (T)v.y);
  }
  __syncthreads();
  const int64_t i0 = ((int64_t)blockIdx.x * DN_TPB + threadIdx.x) * R;
  if (i0 >= n) return;
  T ar[R], ai[R];
#pragma unroll
  for (int r = 0; r < R; ++r) ar[r] = ai[r] = T(0);
  const V* __restrict__ col = reinterpret_cast<const V*>(M + c0 * ld + i0);
  const int64_t vld = ld / R;
  // the diagonal entries of this thread's rows sit in columns i0 .. i0 + R - 1
  const bool diag_here = offdiag && i0 + R > c0 && i0 < c1;
  int64_t j = c0;
  for (; j + 8 <= c1; j += 8) {
    V mv[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mv[q] = col[(size_t)q * vld];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const cx<T> xv = xs[j + q - c0];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T m = (diag_here && j + q == i0 + r) ? T(0) : dn_at<T>(mv[q], r);
        ar[r] = ar[r] + m * xv.x;
        ai[r] = ai[r] + m * xv.y;
      }
    }
    col += (size_t)8 * vld;
  }
  for (; j < c1; ++j, col += vld) {
    const V mv = *col;
    const cx<T> xv = xs[j - c0];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const T m = (diag_here && j == i0 + r) ? T(0) : dn_at<T>(mv, r);
      ar[r] = ar[r] + m * xv.x;
      ai[r] = ai[r] + m * xv.y;
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (i0 + r < n) part[(size_t)blockIdx.y * n + i0 + r] = mk<double>((double)ar[r], (double)ai[r]);
}

// out[i] = sum over chunks of part[chunk][i]: eight lanes per row, lane k summing chunks
// k, k + 8, ... in order, then a fixed shuffle tree over the eight (the same order on
// every run)
constexpr int DN_SUM_LANES = 8;
__global__ void k_dense_sum(const c64* __restrict__ part, int nchunk, int64_t n, c64* out) {
  const int sub = threadIdx.x % DN_SUM_LANES;
  const int64_t rows_per_block = blockDim.x / DN_SUM_LANES;
  for (int64_t i0 = blockIdx.x * rows_per_block; i0 < n; i0 += (int64_t)gridDim.x * rows_per_block) {
    const int64_t i = i0 + threadIdx.x / DN_SUM_LANES;
    double sr = 0.0, si = 0.0;
    if (i < n)
      for (int c = sub; c < nchunk; c += DN_SUM_LANES) {
        const c64 v = part[(size_t)c * n + i];
        sr += v.x;
        si += v.y;
      }
#pragma unroll
    for (int o = DN_SUM_LANES / 2; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o, DN_SUM_LANES);
      si += __shfl_xor_sync(0xffffffffu, si, o, DN_SUM_LANES);
    }
    if (i < n && sub == 0) out[i] = mk<double>(sr, si);
  }
}

// padded leading dimension of an n x n block
int64_t dense_ld(int64_t n) { return std::max<int64_t>(4, (n + 3) / 4 * 4); }

// resident CTAs of the product kernel per SM times the SMs of the current device
// (queried once per device; the kernel's registers and shared memory set it, not a guess)
static int dense_slots(bool fp32) {
  static std::atomic<int> cached[64][2];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::atomic<int>& slot = cached[dev][fp32 ? 1 : 0];
  int c = slot.load();
  if (c == 0) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (fp32)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dense_gemv<float>, DN_TPB, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dense_gemv<double>, DN_TPB, 0);
    cudaGetLastError();
    c = std::max(1, sms) * std::max(1, per);
    slot.store(c);
  }
  return c;
}

// column chunks of an n x n product with R rows per thread: the row tiles times the
// chunks fill one wave of resident CTAs (a partial second wave would double the tail),
// at most DN_CHUNK_MAX columns each
static int dense_chunks_r(int64_t n, int R) {
  if (n <= 0) return 1;
  const int64_t tiles = (n + (int64_t)DN_TPB * R - 1) / ((int64_t)DN_TPB * R);
  int64_t c = dense_slots(R == 4) / tiles;
  const int64_t cmin = (n + DN_CHUNK_MAX - 1) / DN_CHUNK_MAX;
  const int64_t cmax = std::max<int64_t>(1, n / 64);
  if (c > cmax) c = cmax;
  if (c < cmin) c = cmin;
  if (c < 1) c = 1;
  return (int)c;
}
// the larger of the two layouts' chunk counts (the partial-sum scratch serves both)
int dense_chunks(int64_t n) { return std::max(dense_chunks_r(n, 2), dense_chunks_r(n, 4)); }

// out = M x (offdiag: without M's diagonal) for one real block; part holds
// dense_chunks(n) * n entries. Returns the kernels launched.
int dense_apply(const void* M, bool fp32, int64_t n, int64_t ld, const c64* x, int offdiag,
                c64* part, c64* out, cudaStream_t st) {
  if (n <= 0) return 0;
  const int R = fp32 ? 4 : 2;
  const int nc = dense_chunks_r(n, R);
  const int cols = (int)((n + nc - 1) / nc);
  const dim3 grid((unsigned)((n + (int64_t)DN_TPB * R - 1) / ((int64_t)DN_TPB * R)), (unsigned)nc);
  if (fp32)
    k_dense_gemv<float><<<grid, DN_TPB, 0, st>>>((const float*)M, n, ld, x, cols, offdiag, part);
  else
    k_dense_gemv<double><<<grid, DN_TPB, 0, st>>>((const double*)M, n, ld, x, cols, offdiag, part);
  int64_t b = (n + 256 / DN_SUM_LANES - 1) / (256 / DN_SUM_LANES);
  if (b > 152 * 16) b = 152 * 16;
  k_dense_sum<<<(unsigned)b, 256, 0, st>>>(part, nc, n, out);
  return 2;
}

// Complex blocks (the RIS solver's retarded operator, Lp and P times exp(-j beta R)):
// one complex entry per 8 (FP32) or 16 (FP64) bytes, so a thread owns 2 or 1 rows with
// one 16-byte load per column; otherwise as k_dense_gemv.
template <typename T> struct DnCVec;
template <> struct DnCVec<float> { using V = float4; static constexpr int R = 2; };
template <> struct DnCVec<double> { using V = double2; static constexpr int R = 1; };

template <typename T>
__global__ void __launch_bounds__(DN_TPB) k_dense_gemv_c(const cx<T>* __restrict__ M, int64_t n,
                                                         int64_t ld, const c64* __restrict__ x,
                                                         int cols, int offdiag,
                                                         c64* __restrict__ part) {
  using V = typename DnCVec<T>::V;
  constexpr int R = DnCVec<T>::R;
  __shared__ cx<T> xs[DN_CHUNK_MAX];
  const int64_t c0 = (int64_t)blockIdx.y * cols;
  const int64_t c1 = min(c0 + cols, n);
  for (int64_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
    const c64 v = x[j];
    xs[j - c0] = mk<T>((T)v.x, (T)v.y);
  }
  __syncthreads();
  const int64_t i0 = ((int64_t)blockIdx.x * DN_TPB + threadIdx.x) * R;
  if (i0 >= n) return;
  T ar[R], ai[R];
#pragma unroll
  for (int r = 0; r < R; ++r) ar[r] = ai[r] = T(0);
  const V* __restrict__ col = reinterpret_cast<const V*>(M + c0 * ld + i0);
  const int64_t vld = ld / R;
  const bool diag_here = offdiag && i0 + R > c0 && i0 < c1;
  int64_t j = c0;
  for (; j + 8 <= c1; j += 8) {
    V mv[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mv[q] = col[(size_t)q * vld];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const cx<T> xv = xs[j + q - c0];
      const T* e = reinterpret_cast<const T*>(&mv[q]);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const bool z = diag_here && j + q == i0 + r;
        const T mr = z ? T(0) : e[2 * r], mi = z ? T(0) : e[2 * r + 1];
        ar[r] = ar[r] + (mr * xv.x - mi * xv.y);
        ai[r] = ai[r] + (mr * xv.y + mi * xv.x);
      }
    }
    col += (size_t)8 * vld;
  }
  for (; j < c1; ++j, col += vld) {
    const V mv = *col;
    const cx<T> xv = xs[j - c0];
    const T* e = reinterpret_cast<const T*>(&mv);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const bool z = diag_here && j == i0 + r;
      const T mr = z ? T(0) : e[2 * r], mi = z ? T(0) : e[2 * r + 1];
      ar[r] = ar[r] + (mr * xv.x - mi * xv.y);
      ai[r] = ai[r] + (mr * xv.y + mi * xv.x);
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (i0 + r < n) part[(size_t)blockIdx.y * n + i0 + r] = mk<double>((double)ar[r], (double)ai[r]);
}

static int dense_slots_c(bool fp32) {
  static std::atomic<int> cached[64][2];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::atomic<int>& slot = cached[dev][fp32 ? 1 : 0];
  int c = slot.load();
  if (c == 0) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (fp32)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dense_gemv_c<float>, DN_TPB, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dense_gemv_c<double>, DN_TPB, 0);
    cudaGetLastError();
    c = std::max(1, sms) * std::max(1, per);
    slot.store(c);
  }
  return c;
}

static int dense_chunks_c(int64_t n, bool fp32) {
  if (n <= 0) return 1;
  const int R = fp32 ? 2 : 1;
  const int64_t tiles = (n + (int64_t)DN_TPB * R - 1) / ((int64_t)DN_TPB * R);
  int64_t c = dense_slots_c(fp32) / tiles;
  const int64_t cmin = (n + DN_CHUNK_MAX - 1) / DN_CHUNK_MAX;
  const int64_t cmax = std::max<int64_t>(1, n / 64);
  if (c > cmax) c = cmax;
  if (c < cmin) c = cmin;
  if (c < 1) c = 1;
  return (int)c;
}
// partial-sum entries the complex products need (both precisions)
int64_t dense_part_c(int64_t n) {
  return (int64_t)std::max(dense_chunks_c(n, true), dense_chunks_c(n, false)) * std::max<int64_t>(n, 1);
}

// out = M x for a complex block (offdiag: without M's diagonal). Returns the kernels launched.
int dense_apply_c(const void* M, bool fp32, int64_t n, int64_t ld, const c64* x, int offdiag,
                  c64* part, c64* out, cudaStream_t st) {
  if (n <= 0) return 0;
  const int R = fp32 ? 2 : 1;
  const int nc = dense_chunks_c(n, fp32);
  const int cols = (int)((n + nc - 1) / nc);
  const dim3 grid((unsigned)((n + (int64_t)DN_TPB * R - 1) / ((int64_t)DN_TPB * R)), (unsigned)nc);
  if (fp32)
    k_dense_gemv_c<float><<<grid, DN_TPB, 0, st>>>((const c32*)M, n, ld, x, cols, offdiag, part);
  else
    k_dense_gemv_c<double><<<grid, DN_TPB, 0, st>>>((const c64*)M, n, ld, x, cols, offdiag, part);
  int64_t b = (n + 256 / DN_SUM_LANES - 1) / (256 / DN_SUM_LANES);
  if (b > 152 * 16) b = 152 * 16;
  k_dense_sum<<<(unsigned)b, 256, 0, st>>>(part, nc, n, out);
  return 2;
}

// the retarded blocks of one frequency: Mc = M * exp(-j beta R) (FP64) and its FP32 copy
// (iter_solver_QS_S_type.jl:40-52; build_row_vox_Rcc.jl's phase on dense entries)
__global__ void k_dense_phase(const double* __restrict__ M, const double* __restrict__ R,
                              size_t cnt, double beta, c64* Mc, c32* Mc32) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < cnt;
       i += (size_t)gridDim.x * blockDim.x) {
    double s, c;
    sincos(beta * R[i], &s, &c);
    const c64 v = mk<double>(M[i] * c, -M[i] * s);
    Mc[i] = v;
    Mc32[i] = mk<float>((float)v.x, (float)v.y);
  }
}

void dense_phase(const double* M, const double* R, size_t cnt, double beta, c64* Mc, c32* Mc32,
                 cudaStream_t st) {
  size_t b = (cnt + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  k_dense_phase<<<(unsigned)b, 256, 0, st>>>(M, R, cnt, beta, Mc, Mc32);
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
