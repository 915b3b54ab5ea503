// Circulant convolutions of the voxel Lp / P Toeplitz blocks, family-combined.
//
// The operator's circulant blocks act between six lattice families: three face
// families of the P tensor (reference families 12, 34, 56) and three edge
// directions of the Lp tensor. Every P block (three diagonal, three cross blocks
// applied in both directions) is a Toeplitz operator between two face families, and
// all six share one circulant grid L_P, so the P part of an operator application is
//   for each face family g: X_g = FFT3(x_g)            (3 forward transforms)
//   for each frequency:     Y_f = sum_g S_fg X_g       (3x3 Hermitian spectral matrix)
//   for each face family f: y_f = IFFT3(Y_f)           (3 inverse transforms)
// instead of the reference's twelve transform pairs. The Lp blocks are diagonal in
// the edge direction and keep one forward/inverse pair each.
//
// Each 3-D transform runs as passes over one axis at a time on a per-family buffer
// T_f[z][y][kx] (kx fastest, Lx x Ly x nz_f), in place:
//   k_xfwd   gather the family's compact vector through its lattice map, zero pad,
//            forward FFT along x (16 pencils per CTA)
//   k_ypass  forward / inverse FFT along y (16 consecutive kx per CTA)
//   k_zconv3 forward FFT along z of the three face families, 3x3 spectral product,
//            inverse FFT along z (one ky, a kx tile per CTA)
//   k_zconv1 same for one edge family with its real spectrum
//   k_xinv   inverse FFT along x and plain store into the compact output through the
//            lattice map (each compact index belongs to exactly one family)
// Only the occupied lattice octant is transformed in each pass (pruning). Inside a
// pass the first radix group reads global memory straight into registers and the
// last group writes straight back (fft_reg.cuh); in the z passes the last forward
// group, the spectral product and the first inverse group run back to back in
// registers. Shared-memory tiles keep sequences contiguous (element (pos, seq) at
// pos*rs + seq), so the middle groups are bank-conflict free.
// Spectra carry the 1/(Lx*Ly*Lz) normalisation and are stored (ky, kz, kx), kx fastest,
// in the transforms' bit-reversed position order.
#include <mutex>
#include <set>
#include <utility>

#include "ctx.hpp"
#include "fft.cuh"
#include "fft_reg.cuh"

namespace peec {

constexpr int TPB = 256;

// copy W_L[e] = exp(-2 pi i e / L) for e < n from the master table of length twmax
template <typename R>
__device__ void load_tw(cx<R>* dst, const cx<R>* __restrict__ master, int twmax, int L, int n) {
  const int step = twmax / L;
  for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = master[e * step];
}

// --------------------------------------------------------------------------- x passes
// CTA: TY = 16 consecutive y rows of one z plane. Tile element (pos, yy) at
// buf[pos*(TY+1) + yy]; the first/last group threads run along x so map reads and
// output gathers are contiguous.

constexpr int LTY = 4;
constexpr int TY = 1 << LTY;
constexpr int XRS = TY + 1;

template <typename R, int Q>
__device__ __forceinline__ void xfwd_first(const c64* __restrict__ xin,
                                           const int32_t* __restrict__ map, cx<R>* buf,
                                           const AxPlan& p, int y0, int z, int nx, int ny,
                                           const cx<R>* W) {
  constexpr int N = 1 << Q;
  const int lh = p.n - Q;
  const int tasks = TY << lh;
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int k = t & ((1 << lh) - 1);
    const int yy = t >> lh;
    const int y = y0 + yy;
    cx<R> v[N];
    const int32_t* mrow = map + ((size_t)z * ny + y) * nx;
#pragma unroll
    for (int r = 0; r < N; ++r) {
      const int x = k + (r << lh);
      v[r] = mk<R>(0, 0);
      if (y < ny && x < nx) {
        const int idx = mrow[x];
        if (idx >= 0) v[r] = ccast<R>(xin[idx]);
      }
    }
    dft_dif<R, Q>(v);
    if (p.ng > 1) group_twiddle<R, Q, false>(v, k, 0, W);
#pragma unroll
    for (int r = 0; r < N; ++r) buf[(k + (r << lh)) * XRS + yy] = v[r];
  }
}

template <typename R, int Q, bool INV>
__device__ __forceinline__ void x_last_inplace(cx<R>* buf, const AxPlan& p) {
  // the group at the end of the stage order (forward) / its mirror (inverse):
  // contiguous positions, no table twiddles
  constexpr int N = 1 << Q;
  const int tasks = TY << (p.n - Q);
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int yy = t & (TY - 1);
    const int start = (t >> LTY) << Q;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = buf[(start + r) * XRS + yy];
    if (!INV) dft_dif<R, Q>(v);
    else dft_dit<R, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r) buf[(start + r) * XRS + yy] = v[r];
  }
}

template <typename R>
__global__ void __launch_bounds__(TPB) k_xfwd(const c64* __restrict__ xin,
                                              const int32_t* __restrict__ map, cx<R>* T,
                                              AxPlan p, int Ly, int nx, int ny,
                                              const cx<R>* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int Lx = 1 << p.n;
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + Lx;
  const int y0 = blockIdx.x * TY, z = blockIdx.y;
  load_twiddles<R>(W, twm, twmax, Lx);
  __syncthreads();
  qswitch<4>(p.q[0], [&](auto QC) {
    xfwd_first<R, decltype(QC)::value>(xin, map, buf, p, y0, z, nx, ny, W);
  });
  __syncthreads();
  if (p.ng > 1) {
    middle_groups<R, false, LTY>(buf, XRS, p, W);
    qswitch<4>(p.q[p.ng - 1],
               [&](auto QC) { x_last_inplace<R, decltype(QC)::value, false>(buf, p); });
    __syncthreads();
  }
  for (int q = threadIdx.x; q < TY << p.n; q += blockDim.x) {
    const int yy = q >> p.n, kx = q & (Lx - 1);
    const int y = y0 + yy;
    if (y < ny) T[((size_t)z * Ly + y) * Lx + kx] = buf[kx * XRS + yy];
  }
}

template <typename R, int Q>
__device__ __forceinline__ void xinv_last(const cx<R>* buf, c64* yout,
                                          const int32_t* __restrict__ map, const AxPlan& p,
                                          int y0, int z, int nx, int ny, const cx<R>* W) {
  constexpr int N = 1 << Q;
  const int lh = p.n - Q;
  const int tasks = TY << lh;
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int k = t & ((1 << lh) - 1);
    const int yy = t >> lh;
    const int y = y0 + yy;
    if (y >= ny || k >= nx) continue;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = buf[(k + (r << lh)) * XRS + yy];
    if (p.ng > 1) group_twiddle<R, Q, true>(v, k, 0, W);
    dft_dit<R, Q>(v);
    const int32_t* mrow = map + ((size_t)z * ny + y) * nx;
#pragma unroll
    for (int r = 0; r < N; ++r) {
      const int x = k + (r << lh);
      if (x < nx) {
        const int idx = mrow[x];
        if (idx >= 0) yout[idx] = mk<double>((double)v[r].x, (double)v[r].y);
      }
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(TPB) k_xinv(const cx<R>* __restrict__ T, c64* yout,
                                              const int32_t* __restrict__ map, AxPlan p, int Ly,
                                              int nx, int ny, const cx<R>* __restrict__ twm,
                                              int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int Lx = 1 << p.n;
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + Lx;
  const int y0 = blockIdx.x * TY, z = blockIdx.y;
  load_twiddles<R>(W, twm, twmax, Lx);
  for (int q = threadIdx.x; q < TY << p.n; q += blockDim.x) {
    const int yy = q >> p.n, kx = q & (Lx - 1);
    const int y = y0 + yy;
    buf[kx * XRS + yy] = (y < ny) ? T[((size_t)z * Ly + y) * Lx + kx] : mk<R>(0, 0);
  }
  __syncthreads();
  if (p.ng > 1) {
    qswitch<4>(p.q[p.ng - 1],
               [&](auto QC) { x_last_inplace<R, decltype(QC)::value, true>(buf, p); });
    __syncthreads();
    middle_groups<R, true, LTY>(buf, XRS, p, W);
  }
  qswitch<4>(p.q[0], [&](auto QC) {
    xinv_last<R, decltype(QC)::value>(buf, yout, map, p, y0, z, nx, ny, W);
  });
}

// --------------------------------------------------------------------------- column passes
// y and z passes work on columns of TX = 16 consecutive kx: element (pos, col) of the
// tile at buf[pos*TX + col]; global row pos of the column tile at g + pos*gstride.

constexpr int LTX = 4;
constexpr int TX = 1 << LTX;

// forward first group from global rows < n_in (zero beyond), into registers, then the
// tile (or, for a single-group plan, back to global in full)
template <typename R, int Q>
__device__ __forceinline__ void col_first_fwd(const cx<R>* g, size_t gstride, int ncols,
                                              int n_in, cx<R>* buf, const AxPlan& p,
                                              const cx<R>* W, cx<R>* gout) {
  constexpr int N = 1 << Q;
  const int lh = p.n - Q;
  const int tasks = TX << lh;
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int k = t >> LTX;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) {
      const int row = k + (r << lh);
      v[r] = (col < ncols && row < n_in) ? g[row * gstride + col] : mk<R>(0, 0);
    }
    dft_dif<R, Q>(v);
    if (p.ng > 1) {
      group_twiddle<R, Q, false>(v, k, 0, W);
#pragma unroll
      for (int r = 0; r < N; ++r) buf[((k + (r << lh)) << LTX) + col] = v[r];
    } else if (col < ncols) {
#pragma unroll
      for (int r = 0; r < N; ++r) gout[r * gstride + col] = v[r];
    }
  }
}

// forward last group: tile -> global, contiguous positions
template <typename R, int Q>
__device__ __forceinline__ void col_last_fwd(const cx<R>* buf, cx<R>* g, size_t gstride,
                                             int ncols, const AxPlan& p) {
  constexpr int N = 1 << Q;
  const int tasks = TX << (p.n - Q);
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int start = (t >> LTX) << Q;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = buf[((start + r) << LTX) + col];
    dft_dif<R, Q>(v);
    if (col < ncols) {
#pragma unroll
      for (int r = 0; r < N; ++r) g[(start + r) * gstride + col] = v[r];
    }
  }
}

// inverse first group (mirror of the forward last group): global -> tile, or for a
// single-group plan global -> global rows < n_out
template <typename R, int Q>
__device__ __forceinline__ void col_first_inv(const cx<R>* g, size_t gstride, int ncols,
                                              int n_out, cx<R>* buf, const AxPlan& p,
                                              cx<R>* gout) {
  constexpr int N = 1 << Q;
  const int tasks = TX << (p.n - Q);
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int start = (t >> LTX) << Q;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r)
      v[r] = col < ncols ? g[(start + r) * gstride + col] : mk<R>(0, 0);
    dft_dit<R, Q>(v);
    if (p.ng > 1) {
#pragma unroll
      for (int r = 0; r < N; ++r) buf[((start + r) << LTX) + col] = v[r];
    } else if (col < ncols) {
#pragma unroll
      for (int r = 0; r < N; ++r)
        if (start + r < n_out) gout[(start + r) * gstride + col] = v[r];
    }
  }
}

// inverse last group (mirror of the forward first group): tile -> global rows < n_out
template <typename R, int Q>
__device__ __forceinline__ void col_last_inv(const cx<R>* buf, cx<R>* g, size_t gstride,
                                             int ncols, int n_out, const AxPlan& p,
                                             const cx<R>* W) {
  constexpr int N = 1 << Q;
  const int lh = p.n - Q;
  const int tasks = TX << lh;
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int k = t >> LTX;
    if (k >= n_out) continue;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = buf[((k + (r << lh)) << LTX) + col];
    group_twiddle<R, Q, true>(v, k, 0, W);
    dft_dit<R, Q>(v);
    if (col < ncols) {
#pragma unroll
      for (int r = 0; r < N; ++r) {
        const int row = k + (r << lh);
        if (row < n_out) g[row * gstride + col] = v[r];
      }
    }
  }
}

// register-group caps per kernel (see make_plan): x/y passes 16 points at both ends;
// z passes hold three families (P) or one (Lp) at the fused spectral step
template <typename R>
struct QCap {
  static constexpr int XY = 4;
  static constexpr int Z3 = sizeof(R) == 8 ? 2 : 3;
  static constexpr int Z1 = sizeof(R) == 8 ? 3 : 4;
};

// --------------------------------------------------------------------------- y pass
// planes z < nz; rows y < n_in are read (zero padded to Ly), rows y < n_out written
template <typename R, bool INV>
__global__ void __launch_bounds__(TPB) k_ypass(cx<R>* T, int Lx, AxPlan p, int n_in, int n_out,
                                               const cx<R>* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int Ly = 1 << p.n;
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + Ly;
  const int kx0 = blockIdx.x * TX, z = blockIdx.y;
  const int ncols = min(TX, Lx - kx0);
  cx<R>* col = T + (size_t)z * Ly * Lx + kx0;
  load_twiddles<R>(W, twm, twmax, Ly);
  __syncthreads();
  if (!INV) {
    qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(col, (size_t)Lx, ncols, n_in, buf, p, W, col); });
    if (p.ng > 1) {
      __syncthreads();
      middle_groups<R, false, LTX>(buf, TX, p, W);
      qswitch<QCap<R>::XY>(p.q[p.ng - 1], [&](auto QC) { col_last_fwd<R, decltype(QC)::value>(buf, col, (size_t)Lx, ncols, p); });
    }
  } else {
    qswitch<QCap<R>::XY>(p.q[p.ng - 1], [&](auto QC) { col_first_inv<R, decltype(QC)::value>(col, (size_t)Lx, ncols, n_out, buf, p, col); });
    if (p.ng > 1) {
      __syncthreads();
      middle_groups<R, true, LTX>(buf, TX, p, W);
      qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf, col, (size_t)Lx, ncols, n_out, p, W); });
    }
  }
}

// --------------------------------------------------------------------------- z passes

struct PSpec {
  const void* s00;
  const void* s11;
  const void* s22;  // real
  const void* s01;
  const void* s02;
  const void* s12;  // complex
};

// Y_f = sum_g S_fg X_g with S_gf = conj(S_fg), at spectrum index si
template <typename R>
__device__ __forceinline__ void pspec_apply(const PSpec& S, size_t si, cx<R>& a0, cx<R>& a1,
                                            cx<R>& a2) {
  const R* s00 = reinterpret_cast<const R*>(S.s00);
  const R* s11 = reinterpret_cast<const R*>(S.s11);
  const R* s22 = reinterpret_cast<const R*>(S.s22);
  const cx<R>* s01 = reinterpret_cast<const cx<R>*>(S.s01);
  const cx<R>* s02 = reinterpret_cast<const cx<R>*>(S.s02);
  const cx<R>* s12 = reinterpret_cast<const cx<R>*>(S.s12);
  const cx<R> c01 = s01[si], c02 = s02[si], c12 = s12[si];
  const cx<R> b0 = cscale(a0, s00[si]) + c01 * a1 + c02 * a2;
  const cx<R> b1 = cmulc(a0, c01) + cscale(a1, s11[si]) + c12 * a2;
  const cx<R> b2 = cmulc(a0, c02) + cmulc(a1, c12) + cscale(a2, s22[si]);
  a0 = b0;
  a1 = b1;
  a2 = b2;
}

// single-group z transform of all three face families in registers
template <typename R, int Q>
__device__ __forceinline__ void z3_single(cx<R>* T0, cx<R>* T1, cx<R>* T2, int nz0, int nz1,
                                          int nz2, size_t pl, int ncols, const PSpec& S,
                                          size_t sbase, size_t sstride) {
  constexpr int N = 1 << Q;
  for (int col = threadIdx.x; col < TX; col += blockDim.x) {
    if (col >= ncols) continue;
    cx<R> v[3][N];
#pragma unroll
    for (int r = 0; r < N; ++r) {
      v[0][r] = r < nz0 ? T0[r * pl + col] : mk<R>(0, 0);
      v[1][r] = r < nz1 ? T1[r * pl + col] : mk<R>(0, 0);
      v[2][r] = r < nz2 ? T2[r * pl + col] : mk<R>(0, 0);
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) dft_dif<R, Q>(v[f]);
#pragma unroll
    for (int r = 0; r < N; ++r)
      pspec_apply<R>(S, sbase + r * sstride + col, v[0][r], v[1][r], v[2][r]);
#pragma unroll
    for (int f = 0; f < 3; ++f) dft_dit<R, Q>(v[f]);
#pragma unroll
    for (int r = 0; r < N; ++r) {
      if (r < nz0) T0[r * pl + col] = v[0][r];
      if (r < nz1) T1[r * pl + col] = v[1][r];
      if (r < nz2) T2[r * pl + col] = v[2][r];
    }
  }
}

// fused middle step: last forward group of the three families, spectral product,
// first inverse group, tile -> tile (the three tiles are consecutive: tile f at
// buf + f*tsz)
template <typename R, int Q>
__device__ __forceinline__ void z3_fused(cx<R>* buf, size_t tsz, const AxPlan& p, int ncols,
                                         const PSpec& S, size_t sbase, size_t sstride) {
  constexpr int N = 1 << Q;
  const int tasks = TX << (p.n - Q);
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int start = (t >> LTX) << Q;
    cx<R> v[3][N];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
#pragma unroll
      for (int r = 0; r < N; ++r) v[f][r] = buf[f * tsz + ((start + r) << LTX) + col];
      dft_dif<R, Q>(v[f]);
    }
    if (col < ncols) {
#pragma unroll
      for (int r = 0; r < N; ++r)
        pspec_apply<R>(S, sbase + (start + r) * sstride + col, v[0][r], v[1][r], v[2][r]);
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      dft_dit<R, Q>(v[f]);
#pragma unroll
      for (int r = 0; r < N; ++r) buf[f * tsz + ((start + r) << LTX) + col] = v[f][r];
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(TPB, 2) k_zconv3(cx<R>* T0, cx<R>* T1, cx<R>* T2, int nz0, int nz1,
                                                int nz2, PSpec S, int Lx, int Ly, AxPlan p,
                                                const cx<R>* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int Lz = 1 << p.n;
  const size_t tsz = (size_t)Lz << LTX;
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + Lz;  // three tiles, family f at buf + f*tsz
  const int kx0 = blockIdx.x * TX, ky = blockIdx.y;
  const int ncols = min(TX, Lx - kx0);
  const size_t pl = (size_t)Ly * Lx;
  const size_t off = (size_t)ky * Lx + kx0;
  T0 += off;
  T1 += off;
  T2 += off;
  // spectrum index of (ky, kz, kx0 + col) = sbase + kz*Lx + col
  const size_t sbase = (size_t)ky * Lz * Lx + kx0;
  load_twiddles<R>(W, twm, twmax, Lz);
  __syncthreads();
  if (p.ng == 1) {
    qswitch<QCap<R>::Z3>(p.q[0], [&](auto QC) { z3_single<R, decltype(QC)::value>(T0, T1, T2, nz0, nz1, nz2, pl, ncols, S, sbase, (size_t)Lx); });
    return;
  }
  qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(T0, pl, ncols, nz0, buf, p, W, T0); });
  qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(T1, pl, ncols, nz1, buf + tsz, p, W, T1); });
  qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(T2, pl, ncols, nz2, buf + 2 * tsz, p, W, T2); });
  __syncthreads();
  {
    int s = p.q[0];
    for (int g = 1; g + 1 < p.ng; ++g) {
      smem_group_q<R, false, LTX>(buf, TX, p.q[g], p.n, s, W);
      smem_group_q<R, false, LTX>(buf + tsz, TX, p.q[g], p.n, s, W);
      smem_group_q<R, false, LTX>(buf + 2 * tsz, TX, p.q[g], p.n, s, W);
      s += p.q[g];
      __syncthreads();
    }
  }
  qswitch<QCap<R>::Z3>(p.q[p.ng - 1], [&](auto QC) { z3_fused<R, decltype(QC)::value>(buf, tsz, p, ncols, S, sbase, (size_t)Lx); });
  __syncthreads();
  {
    int s = p.n - p.q[p.ng - 1];
    for (int g = p.ng - 2; g >= 1; --g) {
      s -= p.q[g];
      smem_group_q<R, true, LTX>(buf, TX, p.q[g], p.n, s, W);
      smem_group_q<R, true, LTX>(buf + tsz, TX, p.q[g], p.n, s, W);
      smem_group_q<R, true, LTX>(buf + 2 * tsz, TX, p.q[g], p.n, s, W);
      __syncthreads();
    }
  }
  qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf, T0, pl, ncols, nz0, p, W); });
  qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf + tsz, T1, pl, ncols, nz1, p, W); });
  qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf + 2 * tsz, T2, pl, ncols, nz2, p, W); });
}

// one edge family with its real spectrum
template <typename R, int Q>
__device__ __forceinline__ void z1_single(cx<R>* Tg, int nz, size_t pl, int ncols,
                                          const R* __restrict__ s, size_t sbase,
                                          size_t sstride) {
  constexpr int N = 1 << Q;
  for (int col = threadIdx.x; col < TX; col += blockDim.x) {
    if (col >= ncols) continue;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = r < nz ? Tg[r * pl + col] : mk<R>(0, 0);
    dft_dif<R, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = cscale(v[r], s[sbase + r * sstride + col]);
    dft_dit<R, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r)
      if (r < nz) Tg[r * pl + col] = v[r];
  }
}

template <typename R, int Q>
__device__ __forceinline__ void z1_fused(cx<R>* buf, const AxPlan& p, int ncols,
                                         const R* __restrict__ s, size_t sbase, size_t sstride) {
  constexpr int N = 1 << Q;
  const int tasks = TX << (p.n - Q);
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int start = (t >> LTX) << Q;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = buf[((start + r) << LTX) + col];
    dft_dif<R, Q>(v);
    if (col < ncols) {
#pragma unroll
      for (int r = 0; r < N; ++r) v[r] = cscale(v[r], s[sbase + (start + r) * sstride + col]);
    }
    dft_dit<R, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r) buf[((start + r) << LTX) + col] = v[r];
  }
}

template <typename R>
__global__ void __launch_bounds__(TPB) k_zconv1(cx<R>* T0, int nz0, const R* __restrict__ s00,
                                                int Lx, int Ly, AxPlan p,
                                                const cx<R>* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int Lz = 1 << p.n;
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + Lz;
  const int kx0 = blockIdx.x * TX, ky = blockIdx.y;
  const int ncols = min(TX, Lx - kx0);
  const size_t pl = (size_t)Ly * Lx;
  cx<R>* Tg = T0 + (size_t)ky * Lx + kx0;
  const size_t sbase = (size_t)ky * Lz * Lx + kx0;
  load_twiddles<R>(W, twm, twmax, Lz);
  __syncthreads();
  if (p.ng == 1) {
    qswitch<QCap<R>::Z1>(p.q[0], [&](auto QC) { z1_single<R, decltype(QC)::value>(Tg, nz0, pl, ncols, s00, sbase, (size_t)Lx); });
    return;
  }
  qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(Tg, pl, ncols, nz0, buf, p, W, Tg); });
  __syncthreads();
  middle_groups<R, false, LTX>(buf, TX, p, W);
  qswitch<QCap<R>::Z1>(p.q[p.ng - 1], [&](auto QC) { z1_fused<R, decltype(QC)::value>(buf, p, ncols, s00, sbase, (size_t)Lx); });
  __syncthreads();
  middle_groups<R, true, LTX>(buf, TX, p, W);
  qswitch<QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf, Tg, pl, ncols, nz0, p, W); });
}

// --------------------------------------------------------------------------- host side

// Dynamic shared memory above 48 KB needs a per-kernel opt-in. It is set once per
// kernel instantiation to the device maximum (at context set-up, outside any launch
// sequence), so operator applications only launch kernels.
template <typename K>
static int smem_optin(K kernel, size_t bytes) {
  // kernels sharing a signature share K, so the record is keyed by address and device
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  if (bytes > 227 * 1024) {
    set_error("shared memory tile exceeds 227 KB: grid too large for this build");
    return PEEC_ERR_UNSUPPORTED_INTERNAL;
  }
  int dev = 0;
  PEEC_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair((const void*)kernel, dev);
  if (!done.count(key)) {
    int maxsm = 0;
    PEEC_CUDA_TRY(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    PEEC_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm));
    done.insert(key);
  }
  return 0;
}

// radix plans per pass: x/y passes take up to 16 points per register group at both
// ends; the z passes hold 3 families (P) at the fused step, so their last group is
// smaller (FP64 registers are twice as wide)
template <typename R>
struct Plans {
  static AxPlan xy(int n) { return make_plan(n, 4, 4, 4); }
  static AxPlan z3(int n) { return sizeof(R) == 8 ? make_plan(n, 2, 4, 2) : make_plan(n, 3, 4, 3); }
  static AxPlan z1(int n) { return sizeof(R) == 8 ? make_plan(n, 3, 4, 3) : make_plan(n, 4, 4, 4); }
};

template <typename R>
struct Launch {
  static cx<R>* buf(const Family& f) {
    return reinterpret_cast<cx<R>*>(f.T[sizeof(R) == 8 ? 0 : 1]);
  }
  static int xfwd(const Family& f, const c64* xin, const cx<R>* tw, int twmax, cudaStream_t st) {
    const int Lx = f.L[0];
    const size_t sm = sizeof(cx<R>) * (Lx + (size_t)Lx * XRS);
    CTX_CHECK(smem_optin(k_xfwd<R>, sm));
    dim3 g((f.dims[1] + TY - 1) / TY, f.dims[2]);
    k_xfwd<R><<<g, TPB, sm, st>>>(xin, f.map, buf(f), Plans<R>::xy(f.logL[0]), f.L[1], f.dims[0],
                                  f.dims[1], tw, twmax);
    return 0;
  }
  static int xinv(const Family& f, c64* yout, const cx<R>* tw, int twmax, cudaStream_t st) {
    const int Lx = f.L[0];
    const size_t sm = sizeof(cx<R>) * (Lx + (size_t)Lx * XRS);
    CTX_CHECK(smem_optin(k_xinv<R>, sm));
    dim3 g((f.dims[1] + TY - 1) / TY, f.dims[2]);
    k_xinv<R><<<g, TPB, sm, st>>>(buf(f), yout, f.map, Plans<R>::xy(f.logL[0]), f.L[1], f.dims[0],
                                  f.dims[1], tw, twmax);
    return 0;
  }
  template <bool INV>
  static int ypass(const Family& f, const cx<R>* tw, int twmax, cudaStream_t st) {
    const int Ly = f.L[1];
    const size_t sm = sizeof(cx<R>) * (Ly + ((size_t)Ly << LTX));
    CTX_CHECK(smem_optin(k_ypass<R, INV>, sm));
    dim3 g((f.L[0] + TX - 1) / TX, f.dims[2]);
    k_ypass<R, INV><<<g, TPB, sm, st>>>(buf(f), f.L[0], Plans<R>::xy(f.logL[1]),
                                        INV ? Ly : f.dims[1], INV ? f.dims[1] : Ly, tw, twmax);
    return 0;
  }
  static int zconv3(const Family* F, const PSpec& S, const cx<R>* tw, int twmax,
                    cudaStream_t st) {
    const int Lz = F[0].L[2];
    const size_t sm = sizeof(cx<R>) * (Lz + 3 * ((size_t)Lz << LTX));
    CTX_CHECK(smem_optin(k_zconv3<R>, sm));
    dim3 g((F[0].L[0] + TX - 1) / TX, F[0].L[1]);
    k_zconv3<R><<<g, TPB, sm, st>>>(buf(F[0]), buf(F[1]), buf(F[2]), F[0].dims[2], F[1].dims[2],
                                    F[2].dims[2], S, F[0].L[0], F[0].L[1],
                                    Plans<R>::z3(F[0].logL[2]), tw, twmax);
    return 0;
  }
  static int zconv1(const Family& f, const void* s, const cx<R>* tw, int twmax, cudaStream_t st) {
    const int Lz = f.L[2];
    const size_t sm = sizeof(cx<R>) * (Lz + ((size_t)Lz << LTX));
    CTX_CHECK(smem_optin(k_zconv1<R>, sm));
    dim3 g((f.L[0] + TX - 1) / TX, f.L[1]);
    k_zconv1<R><<<g, TPB, sm, st>>>(buf(f), f.dims[2], reinterpret_cast<const R*>(s), f.L[0],
                                    f.L[1], Plans<R>::z1(f.logL[2]), tw, twmax);
    return 0;
  }
};

// ev (nullable): 6 events bracketing the five pass classes
template <typename R>
static int conv_all_t(const Family* F, int nfam, const Spectrum* spec, const c64* x, c64* LpI,
                      c64* PQ, int64_t m, const cx<R>* tw, int twmax, cudaStream_t st,
                      cudaEvent_t* ev) {
  using Lc = Launch<R>;
  const int p = sizeof(R) == 8 ? 0 : 1;
  if (ev) cudaEventRecord(ev[0], st);
  for (int f = 0; f < nfam; ++f)
    if (F[f].active) CTX_CHECK(Lc::xfwd(F[f], F[f].lp ? x : x + m, tw, twmax, st));
  if (ev) cudaEventRecord(ev[1], st);
  for (int f = 0; f < nfam; ++f)
    if (F[f].active) CTX_CHECK(Lc::template ypass<false>(F[f], tw, twmax, st));
  if (ev) cudaEventRecord(ev[2], st);
  PSpec S{spec[0].d[p], spec[1].d[p], spec[2].d[p], spec[3].d[p], spec[4].d[p], spec[5].d[p]};
  CTX_CHECK(Lc::zconv3(F, S, tw, twmax, st));
  for (int f = 3; f < nfam; ++f)
    if (F[f].active) CTX_CHECK(Lc::zconv1(F[f], spec[3 + f].d[p], tw, twmax, st));
  if (ev) cudaEventRecord(ev[3], st);
  for (int f = 0; f < nfam; ++f)
    if (F[f].active) CTX_CHECK(Lc::template ypass<true>(F[f], tw, twmax, st));
  if (ev) cudaEventRecord(ev[4], st);
  for (int f = 0; f < nfam; ++f)
    if (F[f].active) CTX_CHECK(Lc::xinv(F[f], F[f].lp ? LpI : PQ, tw, twmax, st));
  if (ev) cudaEventRecord(ev[5], st);
  return 0;
}

int conv_all(const Family* F, int nfam, const Spectrum* spec, const c64* x, c64* LpI, c64* PQ,
             int64_t m, int prec, const void* tw64, const void* tw32, int twmax, cudaStream_t st,
             cudaEvent_t* ev) {
  if (prec == 0)
    return conv_all_t<double>(F, nfam, spec, x, LpI, PQ, m, reinterpret_cast<const c64*>(tw64),
                              twmax, st, ev);
  return conv_all_t<float>(F, nfam, spec, x, LpI, PQ, m, reinterpret_cast<const c32*>(tw32), twmax,
                           st, ev);
}


// --------------------------------------------------------------------------- spectra
// spectra: embed the generating row as a (possibly non-symmetric) circulant kernel,
// forward-FFT it with the same DIF transforms, fold the 1/(Lx*Ly*Lz) scale
// ------------------------------------------------------------------------------------

struct EmbedDim {
  int L, na, nb, s, o, M;
};

__device__ __forceinline__ int embed_index(int j, const EmbedDim& d) {
  // offset e of circulant slot j: e = j for j < na, e = j - L for j > L - nb
  int e;
  if (j < d.na) e = j;
  else if (j > d.L - d.nb) e = j - d.L;
  else return -1;
  int t = d.s * e + d.o;
  t = t < 0 ? -t : t;
  return t < d.M ? t : -1;
}

__global__ void k_embed(const double* __restrict__ row, c64* out, EmbedDim dx, EmbedDim dy,
                        EmbedDim dz) {
  const size_t total = (size_t)dx.L * dy.L * dz.L;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const int jz = p % dz.L;
    const int jy = (p / dz.L) % dy.L;
    const int jx = p / ((size_t)dz.L * dy.L);
    const int ix = embed_index(jx, dx), iy = embed_index(jy, dy), iz = embed_index(jz, dz);
    double v = 0.0;
    if (ix >= 0 && iy >= 0 && iz >= 0) v = row[((size_t)iz * dy.M + iy) * dx.M + ix];
    out[p] = mk<double>(v, 0.0);
  }
}

// forward DIF along one axis of a (Lx,Ly,Lz) array with z fastest. For axis 2 the
// pencils are contiguous; for axes 0/1 a CTA takes TZ consecutive pencils.
template <int TZ>
__global__ void k_fft_axis(c64* data, int Lx, int Ly, int Lz, int axis, int logL,
                           const c64* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int L = axis == 0 ? Lx : (axis == 1 ? Ly : Lz);
  c64* W = reinterpret_cast<c64*>(smem_raw);
  c64* buf = W + (L / 2 > 0 ? L / 2 : 1);
  load_tw<double>(W, twm, twmax, L, L / 2);
  if (axis == 2) {
    // TZ pencils: rows of length Lz
    const size_t row0 = (size_t)blockIdx.x * TZ;
    const size_t nrows = (size_t)Lx * Ly;
    const int sst = L + 1;
    for (int p = threadIdx.x; p < TZ * L; p += blockDim.x) {
      const int rr = p / L, z = p - rr * L;
      buf[rr * sst + z] = (row0 + rr < nrows) ? data[(row0 + rr) * L + z] : mk<double>(0, 0);
    }
    __syncthreads();
    block_fft<double, false, false>(buf, TZ, sst, 1, logL, W);
    for (int p = threadIdx.x; p < TZ * L; p += blockDim.x) {
      const int rr = p / L, z = p - rr * L;
      if (row0 + rr < nrows) data[(row0 + rr) * L + z] = buf[rr * sst + z];
    }
  } else {
    // pencils along x or y: take TZ consecutive z at fixed (other index)
    const int nzb = (Lz + TZ - 1) / TZ;
    const int zb = blockIdx.x % nzb;
    const int other = blockIdx.x / nzb;  // y (axis 0) or x (axis 1)
    const size_t stride = axis == 0 ? (size_t)Ly * Lz : (size_t)Lz;
    const size_t base = axis == 0 ? (size_t)other * Lz : (size_t)other * Ly * Lz;
    for (int p = threadIdx.x; p < TZ * L; p += blockDim.x) {
      const int j = p / TZ, zz = p - j * TZ;
      const int z = zb * TZ + zz;
      buf[zz + j * TZ] = (z < Lz) ? data[base + j * stride + z] : mk<double>(0, 0);
    }
    __syncthreads();
    block_fft<double, false, true>(buf, TZ, 1, TZ, logL, W);
    for (int p = threadIdx.x; p < TZ * L; p += blockDim.x) {
      const int j = p / TZ, zz = p - j * TZ;
      const int z = zb * TZ + zz;
      if (z < Lz) data[base + j * stride + z] = buf[zz + j * TZ];
    }
  }
}

// full (x,y,z; z fastest) -> stored (ky, kz, kx; kx fastest), scaled, real part only for
// symmetric kernels, FP64 and FP32 copies
__global__ void k_spec_store(const c64* __restrict__ full, void* d64, void* d32, int Lx, int Ly,
                             int Lz, int is_complex, double scale) {
  const size_t n = (size_t)Lx * Ly * Lz;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < n;
       o += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(o % Lx);
    const size_t r = o / Lx;
    const int kz = (int)(r % Lz), ky = (int)(r / Lz);
    const c64 v = full[((size_t)kx * Ly + ky) * Lz + kz];
    if (is_complex) {
      reinterpret_cast<c64*>(d64)[o] = mk<double>(v.x * scale, v.y * scale);
      reinterpret_cast<c32*>(d32)[o] = mk<float>((float)(v.x * scale), (float)(v.y * scale));
    } else {
      reinterpret_cast<double*>(d64)[o] = v.x * scale;
      reinterpret_cast<float*>(d32)[o] = (float)(v.x * scale);
    }
  }
}

int spectrum_build(Spectrum& S, const double* d_row, const int M[3], const int na[3],
                   const int nb[3], const int sdim[3], const int odim[3], int symmetric,
                   const void* tw64, int twmax, cudaStream_t st) {
  // the kernel embedding of a generating row at S.L, forward-transformed in place
  const size_t n = (size_t)S.L[0] * S.L[1] * S.L[2];
  c64* full = nullptr;
  PEEC_CUDA_TRY(cudaMallocAsync(&full, n * sizeof(c64), st));
  EmbedDim d[3];
  for (int i = 0; i < 3; ++i) d[i] = EmbedDim{S.L[i], na[i], nb[i], sdim[i], odim[i], M[i]};
  k_embed<<<1184, 256, 0, st>>>(d_row, full, d[0], d[1], d[2]);
  const c64* tw = reinterpret_cast<const c64*>(tw64);
  constexpr int TZ = 8;
  for (int axis = 2; axis >= 0; --axis) {
    const int L = S.L[axis];
    const int logL = ilog2(L);
    if (logL == 0) continue;
    size_t sm = sizeof(c64) * ((L / 2) + (size_t)TZ * (L + 1));
    unsigned grid = axis == 2 ? (unsigned)((S.L[0] * (size_t)S.L[1] + TZ - 1) / TZ)
                              : (unsigned)(((S.L[2] + TZ - 1) / TZ) * (axis == 0 ? S.L[1] : S.L[0]));
    if (sm > 48 * 1024)
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_fft_axis<TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sm));
    k_fft_axis<TZ><<<grid, 256, sm, st>>>(full, S.L[0], S.L[1], S.L[2], axis, logL, tw, twmax);
  }
  S.is_complex = symmetric ? 0 : 1;
  const size_t es64 = S.is_complex ? sizeof(c64) : sizeof(double);
  const size_t es32 = S.is_complex ? sizeof(c32) : sizeof(float);
  if (!S.d[0]) PEEC_CUDA_TRY(cudaMalloc(&S.d[0], n * es64));
  if (!S.d[1]) PEEC_CUDA_TRY(cudaMalloc(&S.d[1], n * es32));
  k_spec_store<<<1184, 256, 0, st>>>(full, S.d[0], S.d[1], S.L[0], S.L[1], S.L[2], S.is_complex,
                                     1.0 / (double)n);
  PEEC_CUDA_TRY(cudaGetLastError());
  PEEC_CUDA_TRY(cudaFreeAsync(full, st));
  return 0;
}

}  // namespace peec
