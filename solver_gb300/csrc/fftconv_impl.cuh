// Pass kernels and launch sequence of the circulant convolutions, templated on the
// arithmetic (float, double, float-float); each arithmetic is instantiated in its own
// translation unit (fftconv_f32.cu, fftconv_f64.cu, fftconv_ff.cu) so they compile in
// parallel. The pipeline itself is described in fftconv.cu.
#pragma once
#include <mutex>
#include <set>
#include <type_traits>
#include <utility>

#include "ctx.hpp"
#include "fft_reg.cuh"
#include "tma.cuh"

namespace peec {

constexpr int TPB = 256;
// z passes: 128 threads, so that with Lz = 128 every phase splits evenly (first and
// last groups 3 x 16 columns x 8 pencils, fused step 16 x 16) and four CTAs share an SM
constexpr int ZTPB = 128;

// Family buffers stream through each pass once: loads and stores carry the streaming
// (evict-first) cache hint, so the L2 keeps the spectra and twiddles the passes reuse.
template <typename R>
struct StreamVec;
template <>
struct StreamVec<float> {
  using T = float2;
};
template <>
struct StreamVec<double> {
  using T = double2;
};
template <>
struct StreamVec<ff> {
  using T = float4;
};
template <typename R>
__device__ __forceinline__ cx<R> ld_stream(const cx<R>* p) {
  using V = typename StreamVec<R>::T;
  const V v = __ldcs(reinterpret_cast<const V*>(p));
  return *reinterpret_cast<const cx<R>*>(&v);
}
template <typename R>
__device__ __forceinline__ void st_stream(cx<R>* p, const cx<R>& x) {
  using V = typename StreamVec<R>::T;
  __stcs(reinterpret_cast<V*>(p), *reinterpret_cast<const V*>(&x));
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

// One launch runs a pass over every active family: the CTAs of family i are
// [cta0, cta0 + gx * gy) of the 1-D grid, laid out as that family's own gx x gy grid.
// Separate launches per family left each pass a train of partial waves (at 128x128x64 a
// family's x pass is under one wave of CTAs) with a ramp-up and tail each.
template <typename R>
struct FamPass {
  cx<R>* T;             // family buffer
  const int32_t* map;   // x passes: lattice map
  c64* io;              // x passes: compact input (forward) / output (inverse)
  AxPlan p;             // transform plan along the pass axis
  int L_other;          // x passes: Ly; y passes: Lx
  int a, b;             // x passes: lattice nx, ny; y passes: rows read, rows written
  int gx;               // CTAs along the family grid's first axis
  int cta0;             // first CTA of the family
};
constexpr int kMaxFam = 6;
template <typename R>
struct PassSet {
  int nf;
  FamPass<R> f[kMaxFam];
};

// this CTA's family, and its (x, y) block index in that family's grid
template <typename R>
__device__ __forceinline__ FamPass<R> pick_family(const PassSet<R>& s, int& bx, int& by) {
  const int b = blockIdx.x;
  FamPass<R> F = s.f[0];
#pragma unroll
  for (int i = 1; i < kMaxFam; ++i)
    if (i < s.nf && b >= s.f[i].cta0) F = s.f[i];
  const int lb = b - F.cta0;
  bx = lb % F.gx;
  by = lb / F.gx;
  return F;
}

template <typename R>
__global__ void __launch_bounds__(TPB) k_xfwd(PassSet<R> s, const cx<R>* __restrict__ twm,
                                              int twmax) {
  extern __shared__ unsigned char smem_raw[];
  int bx, by;
  const FamPass<R> F = pick_family(s, bx, by);
  const c64* __restrict__ xin = F.io;
  const int32_t* __restrict__ map = F.map;
  cx<R>* T = F.T;
  const AxPlan& p = F.p;
  const int Ly = F.L_other, nx = F.a, ny = F.b;
  const int Lx = 1 << p.n;
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + Lx;
  const int y0 = bx * TY, z = by;
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
    if (y < ny) st_stream(T + ((size_t)z * Ly + y) * Lx + kx, buf[kx * XRS + yy]);
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
__global__ void __launch_bounds__(TPB) k_xinv(PassSet<R> s, const cx<R>* __restrict__ twm,
                                              int twmax) {
  extern __shared__ unsigned char smem_raw[];
  int bx, by;
  const FamPass<R> F = pick_family(s, bx, by);
  const cx<R>* __restrict__ T = F.T;
  c64* yout = F.io;
  const int32_t* __restrict__ map = F.map;
  const AxPlan& p = F.p;
  const int Ly = F.L_other, nx = F.a, ny = F.b;
  const int Lx = 1 << p.n;
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + Lx;
  const int y0 = bx * TY, z = by;
  load_twiddles<R>(W, twm, twmax, Lx);
  for (int q = threadIdx.x; q < TY << p.n; q += blockDim.x) {
    const int yy = q >> p.n, kx = q & (Lx - 1);
    const int y = y0 + yy;
    buf[kx * XRS + yy] = (y < ny) ? ld_stream(T + ((size_t)z * Ly + y) * Lx + kx) : mk<R>(0, 0);
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
      v[r] = (col < ncols && row < n_in) ? ld_stream(g + row * gstride + col) : mk<R>(0, 0);
    }
    dft_dif<R, Q>(v);
    if (p.ng > 1) {
      group_twiddle<R, Q, false>(v, k, 0, W);
#pragma unroll
      for (int r = 0; r < N; ++r) buf[((k + (r << lh)) << LTX) + col] = v[r];
    } else if (col < ncols) {
#pragma unroll
      for (int r = 0; r < N; ++r) st_stream(gout + r * gstride + col, v[r]);
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
      for (int r = 0; r < N; ++r) st_stream(g + (start + r) * gstride + col, v[r]);
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
      v[r] = col < ncols ? ld_stream(g + (start + r) * gstride + col) : mk<R>(0, 0);
    dft_dit<R, Q>(v);
    if (p.ng > 1) {
#pragma unroll
      for (int r = 0; r < N; ++r) buf[((start + r) << LTX) + col] = v[r];
    } else if (col < ncols) {
#pragma unroll
      for (int r = 0; r < N; ++r)
        if (start + r < n_out) st_stream(gout + (start + r) * gstride + col, v[r]);
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
        if (row < n_out) st_stream(g + row * gstride + col, v[r]);
      }
    }
  }
}

// register-group caps per kernel (see make_plan): x/y passes 16 points at both ends;
// z passes hold three families (P) or one (Lp) at the fused spectral step
template <typename R>
struct QCap {
  static constexpr bool wide = sizeof(R) == 8;  // double and float-float registers
  static constexpr int XY = 4;
  static constexpr int Z3 = wide ? 2 : 3;
  static constexpr int Z1 = wide ? 3 : 4;
};
// buffers and spectra: FP32 passes use the FP32 copies, FP64 and float-float the FP64 ones
template <typename R>
constexpr int slot_of() {
  return std::is_same<R, float>::value ? 1 : 0;
}

// --------------------------------------------------------------------------- y pass
// planes z < nz; rows y < n_in are read (zero padded to Ly), rows y < n_out written
template <typename R, bool INV>
__global__ void __launch_bounds__(TPB) k_ypass(PassSet<R> s, const cx<R>* __restrict__ twm,
                                               int twmax) {
  extern __shared__ unsigned char smem_raw[];
  int bx, by;
  const FamPass<R> F = pick_family(s, bx, by);
  cx<R>* T = F.T;
  const AxPlan& p = F.p;
  const int Lx = F.L_other, n_in = F.a, n_out = F.b;
  const int Ly = 1 << p.n;
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + Ly;
  const int kx0 = bx * TX, z = by;
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

// The six P spectra: full form (diagonal blocks real, cross blocks complex, in the pass's
// storage precision) and octant form (real R, FP64) with the cross blocks' half-sample
// shifts and the face grid's phase tables E_a[p] = exp(-i*pi*k/L_a), k the signed
// frequency of position p. In octant form a cross spectrum is R times the product of
// E_a (shift +1) or conj(E_a) (shift -1) over its shifted axes. The FP32 and FP64 passes
// read the full form (coalesced); the float-float passes read the octant (an eighth of
// the FP64 bytes, and FP32-pipe arithmetic for the phases).
struct PSpec {
  const void* f00;
  const void* f11;
  const void* f22;
  const void* f01;
  const void* f02;
  const void* f12;
  const void* o00;
  const void* o11;
  const void* o22;
  const void* o01;
  const void* o02;
  const void* o12;
  const void* ex;
  const void* ey;
  const void* ez;
  int c01[3], c02[3], c12[3];
  // staged FP32 z pass: y/z-folded R (00, 11, 22, 01, 02, 12) and FP32 phase tables
  const float* y[6];
  const c32* ex32;
  const c32* ey32;
  const c32* ez32;
};

template <typename R>
constexpr bool octant_spectra() {
  return std::is_same<R, ff>::value;
}

// storage type of the spectra a pass of arithmetic type R reads: the float-float
// passes split the FP64 spectra on load
template <typename R>
struct SpecOf {
  using T = R;
};
template <>
struct SpecOf<ff> {
  using T = double;
};
template <typename R>
__device__ __forceinline__ R spec_re(const void* p, size_t i) {
  return R(reinterpret_cast<const typename SpecOf<R>::T*>(p)[i]);
}
template <typename R>
__device__ __forceinline__ cx<R> spec_cx(const void* p, size_t i) {
  const auto v = reinterpret_cast<const cx<typename SpecOf<R>::T>*>(p)[i];
  return mk<R>(R(v.x), R(v.y));
}

__device__ __forceinline__ int brevn(int v, int n) {
  return n ? (int)(__brev((unsigned)v) >> (32 - n)) : 0;
}
// octant index of the frequency at DIF position p of a length-2^n axis
__device__ __forceinline__ int fold_pos(int p, int n) {
  const int k = brevn(p, n), L = 1 << n;
  return k <= (L >> 1) ? k : L - k;
}

// Spectrum addressing of one z-pass CTA (fixed ky, kx tile). Full form: (ky, kz, kx0+col)
// at sbase + kz*Lx + col. Octant form: entry (fy, fz, fx) at (fy*oz + fz)*ox + fx with
// o_a = L_a/2 + 1.
struct OctIdx {
  size_t rowbase;  // fy * oz * ox
  size_t sbase;    // ky * Lz * Lx + kx0
  int Lx, ox, nx, nz, kx0;
  __device__ __forceinline__ size_t at(int col, int pz) const {
    return rowbase + (size_t)fold_pos(pz, nz) * ox + fold_pos(kx0 + col, nx);
  }
  __device__ __forceinline__ size_t full(int col, int pz) const {
    return sbase + (size_t)pz * Lx + col;
  }
};

__device__ __forceinline__ OctIdx make_octidx(int Lx, int Ly, int Lz, int kx0, int ky) {
  OctIdx o;
  o.Lx = Lx;
  o.nx = ilog2(Lx);
  o.nz = ilog2(Lz);
  o.ox = Lx / 2 + 1;
  o.kx0 = kx0;
  o.rowbase = (size_t)fold_pos(ky, ilog2(Ly)) * (Lz / 2 + 1) * o.ox;
  o.sbase = (size_t)ky * Lz * Lx + kx0;
  return o;
}

template <typename R>
__device__ __forceinline__ cx<R> shift_phase(const int c[3], const cx<R>& ex, const cx<R>& ey,
                                             const cx<R>& ez) {
  cx<R> f = mk<R>(1, 0);
  if (c[0]) f = c[0] > 0 ? f * ex : cmulc(f, ex);
  if (c[1]) f = c[1] > 0 ? f * ey : cmulc(f, ey);
  if (c[2]) f = c[2] > 0 ? f * ez : cmulc(f, ez);
  return f;
}

// Y_f = sum_g S_fg X_g with S_gf = conj(S_fg), at the frequency of (column col, z
// position pz) of the CTA; ex / ey the CTA's x (per column) and y phases
template <typename R>
__device__ __forceinline__ void pspec_apply(const PSpec& S, const OctIdx& O, int col, int pz,
                                            const cx<R>& ex, const cx<R>& ey, cx<R>& a0,
                                            cx<R>& a1, cx<R>& a2) {
  cx<R> c01, c02, c12;
  R d00, d11, d22;
  if constexpr (octant_spectra<R>()) {
    const size_t oi = O.at(col, pz);
    const cx<R> ez = spec_cx<R>(S.ez, pz);
    c01 = cscale(shift_phase<R>(S.c01, ex, ey, ez), spec_re<R>(S.o01, oi));
    c02 = cscale(shift_phase<R>(S.c02, ex, ey, ez), spec_re<R>(S.o02, oi));
    c12 = cscale(shift_phase<R>(S.c12, ex, ey, ez), spec_re<R>(S.o12, oi));
    d00 = spec_re<R>(S.o00, oi);
    d11 = spec_re<R>(S.o11, oi);
    d22 = spec_re<R>(S.o22, oi);
  } else {
    const size_t si = O.full(col, pz);
    c01 = spec_cx<R>(S.f01, si);
    c02 = spec_cx<R>(S.f02, si);
    c12 = spec_cx<R>(S.f12, si);
    d00 = spec_re<R>(S.f00, si);
    d11 = spec_re<R>(S.f11, si);
    d22 = spec_re<R>(S.f22, si);
  }
  const cx<R> b0 = cscale(a0, d00) + c01 * a1 + c02 * a2;
  const cx<R> b1 = cmulc(a0, c01) + cscale(a1, d11) + c12 * a2;
  const cx<R> b2 = cmulc(a0, c02) + cmulc(a1, c12) + cscale(a2, d22);
  a0 = b0;
  a1 = b1;
  a2 = b2;
}

// the x and y phases of a column / the CTA (octant form only)
template <typename R>
__device__ __forceinline__ cx<R> phase_at(const void* table, int p) {
  if constexpr (octant_spectra<R>()) return spec_cx<R>(table, p);
  else return mk<R>(1, 0);
}

// single-group z transform of all three face families in registers
template <typename R, int Q>
__device__ __forceinline__ void z3_single(cx<R>* T0, cx<R>* T1, cx<R>* T2, int nz0, int nz1,
                                          int nz2, size_t pl, int ncols, const PSpec& S,
                                          const OctIdx& O, const cx<R>& ey) {
  constexpr int N = 1 << Q;
  for (int col = threadIdx.x; col < TX; col += blockDim.x) {
    if (col >= ncols) continue;
    const cx<R> ex = phase_at<R>(S.ex, O.kx0 + col);
    cx<R> v[3][N];
#pragma unroll
    for (int r = 0; r < N; ++r) {
      v[0][r] = r < nz0 ? ld_stream(T0 + r * pl + col) : mk<R>(0, 0);
      v[1][r] = r < nz1 ? ld_stream(T1 + r * pl + col) : mk<R>(0, 0);
      v[2][r] = r < nz2 ? ld_stream(T2 + r * pl + col) : mk<R>(0, 0);
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) dft_dif<R, Q>(v[f]);
#pragma unroll
    for (int r = 0; r < N; ++r) pspec_apply<R>(S, O, col, r, ex, ey, v[0][r], v[1][r], v[2][r]);
#pragma unroll
    for (int f = 0; f < 3; ++f) dft_dit<R, Q>(v[f]);
#pragma unroll
    for (int r = 0; r < N; ++r) {
      if (r < nz0) st_stream(T0 + r * pl + col, v[0][r]);
      if (r < nz1) st_stream(T1 + r * pl + col, v[1][r]);
      if (r < nz2) st_stream(T2 + r * pl + col, v[2][r]);
    }
  }
}

// fused middle step: last forward group of the three families, spectral product,
// first inverse group, tile -> tile (the three tiles are consecutive: tile f at
// buf + f*tsz)
template <typename R, int Q>
__device__ __forceinline__ void z3_fused(cx<R>* buf, size_t tsz, const AxPlan& p, int ncols,
                                         const PSpec& S, const OctIdx& O, const cx<R>& ey) {
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
      const cx<R> ex = phase_at<R>(S.ex, O.kx0 + col);
#pragma unroll
      for (int r = 0; r < N; ++r)
        pspec_apply<R>(S, O, col, start + r, ex, ey, v[0][r], v[1][r], v[2][r]);
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      dft_dit<R, Q>(v[f]);
#pragma unroll
      for (int r = 0; r < N; ++r) buf[f * tsz + ((start + r) << LTX) + col] = v[f][r];
    }
  }
}

// group size QFIX when the kernel is specialised for it (plans of the common lengths),
// else the runtime value through qswitch
template <int QFIX, int CAP, typename F>
__device__ __forceinline__ void qpick(int q, F&& f) {
  if constexpr (QFIX > 0) f(qconst<QFIX>{});
  else qswitch<CAP>(q, f);
}

// Q0 / QL > 0: instantiation for plans whose first / last groups have those sizes (only
// that register code is compiled: smaller kernels, fewer registers); 0: any plan
template <typename R, int Q0 = 0, int QL = 0>
__global__ void __launch_bounds__(ZTPB, 4) k_zconv3(cx<R>* T0, cx<R>* T1, cx<R>* T2, int nz0, int nz1,
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
  const OctIdx O = make_octidx(Lx, Ly, Lz, kx0, ky);
  const cx<R> ey = phase_at<R>(S.ey, ky);
  load_twiddles<R>(W, twm, twmax, Lz);
  __syncthreads();
  if constexpr (Q0 == 0) {
    if (p.ng == 1) {
      qswitch<QCap<R>::Z3>(p.q[0], [&](auto QC) { z3_single<R, decltype(QC)::value>(T0, T1, T2, nz0, nz1, nz2, pl, ncols, S, O, ey); });
      return;
    }
  }
  qpick<Q0, QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(T0, pl, ncols, nz0, buf, p, W, T0); });
  qpick<Q0, QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(T1, pl, ncols, nz1, buf + tsz, p, W, T1); });
  qpick<Q0, QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(T2, pl, ncols, nz2, buf + 2 * tsz, p, W, T2); });
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
  qpick<QL, QCap<R>::Z3>(p.q[p.ng - 1], [&](auto QC) { z3_fused<R, decltype(QC)::value>(buf, tsz, p, ncols, S, O, ey); });
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
  qpick<Q0, QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf, T0, pl, ncols, nz0, p, W); });
  qpick<Q0, QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf + tsz, T1, pl, ncols, nz1, p, W); });
  qpick<Q0, QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf + 2 * tsz, T2, pl, ncols, nz2, p, W); });
}

// one edge family with its real spectrum
template <typename R, int Q>
__device__ __forceinline__ void z1_single(cx<R>* Tg, int nz, size_t pl, int ncols,
                                          const void* __restrict__ s, const OctIdx& O) {
  constexpr int N = 1 << Q;
  for (int col = threadIdx.x; col < TX; col += blockDim.x) {
    if (col >= ncols) continue;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = r < nz ? ld_stream(Tg + r * pl + col) : mk<R>(0, 0);
    dft_dif<R, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r)
      v[r] = cscale(v[r], spec_re<R>(s, octant_spectra<R>() ? O.at(col, r) : O.full(col, r)));
    dft_dit<R, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r)
      if (r < nz) st_stream(Tg + r * pl + col, v[r]);
  }
}

template <typename R, int Q>
__device__ __forceinline__ void z1_fused(cx<R>* buf, const AxPlan& p, int ncols,
                                         const void* __restrict__ s, const OctIdx& O) {
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
      for (int r = 0; r < N; ++r)
        v[r] = cscale(v[r], spec_re<R>(s, octant_spectra<R>() ? O.at(col, start + r)
                                                              : O.full(col, start + r)));
    }
    dft_dit<R, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r) buf[((start + r) << LTX) + col] = v[r];
  }
}

template <typename R, int Q0 = 0, int QL = 0>
__global__ void __launch_bounds__(ZTPB, 4) k_zconv1(cx<R>* T0, int nz0, const void* __restrict__ s00,
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
  const OctIdx O = make_octidx(Lx, Ly, Lz, kx0, ky);
  load_twiddles<R>(W, twm, twmax, Lz);
  __syncthreads();
  if constexpr (Q0 == 0) {
    if (p.ng == 1) {
      qswitch<QCap<R>::Z1>(p.q[0], [&](auto QC) { z1_single<R, decltype(QC)::value>(Tg, nz0, pl, ncols, s00, O); });
      return;
    }
  }
  qpick<Q0, QCap<R>::XY>(p.q[0], [&](auto QC) { col_first_fwd<R, decltype(QC)::value>(Tg, pl, ncols, nz0, buf, p, W, Tg); });
  __syncthreads();
  middle_groups<R, false, LTX>(buf, TX, p, W);
  qpick<QL, QCap<R>::Z1>(p.q[p.ng - 1], [&](auto QC) { z1_fused<R, decltype(QC)::value>(buf, p, ncols, s00, O); });
  __syncthreads();
  middle_groups<R, true, LTX>(buf, TX, p, W);
  qpick<Q0, QCap<R>::XY>(p.q[0], [&](auto QC) { col_last_inv<R, decltype(QC)::value>(buf, Tg, pl, ncols, nz0, p, W); });
}

// --------------------------------------------------------------------------- staged z passes
// FP32 z passes over persistent CTAs that walk the tiles (one ky row, 16 kx columns) in a
// grid-stride loop. One warp stages the next tile's occupied z rows of every family into a
// shared-memory buffer with bulk asynchronous copies (cp.async.bulk, 128-byte rows,
// mbarrier completion) while the CTA computes the current tile, so HBM reads overlap the
// FFT arithmetic instead of stalling it. The first group reads the staged rows; the
// middle, fused and last groups are those of k_zconv3 / k_zconv1. Spectra come from the
// y/z-folded FP32 tables (Spectrum::yz32), which stay largely resident in L2.
// Bounded waits: a copy wait that runs out sets *err, waits once more (bounded) for the
// copies in flight and ends the CTA.

constexpr int ZWAIT_LIMIT = 1 << 20;

// spectrum index of the tile's column col at z position pz in the y/z-folded tables
struct YzIdx {
  size_t rowbase;  // fold(ky) * (Lz/2 + 1) * Lx + kx0
  int Lx, nz;
  __device__ __forceinline__ size_t at(int col, int pz) const {
    return rowbase + (size_t)fold_pos(pz, nz) * Lx + col;
  }
};

__device__ __forceinline__ YzIdx make_yzidx(int Lx, int Ly, int Lz, int kx0, int ky) {
  YzIdx y;
  y.Lx = Lx;
  y.nz = ilog2(Lz);
  y.rowbase = (size_t)fold_pos(ky, ilog2(Ly)) * (Lz / 2 + 1) * Lx + kx0;
  return y;
}

__device__ __forceinline__ void pspec_apply_yz(const PSpec& S, const YzIdx& Y, int col, int pz,
                                               const c32& ex, const c32& ey, c32& a0, c32& a1,
                                               c32& a2) {
  const size_t i = Y.at(col, pz);
  const c32 ez = S.ez32[pz];
  const c32 c01 = cscale(shift_phase<float>(S.c01, ex, ey, ez), __ldg(S.y[3] + i));
  const c32 c02 = cscale(shift_phase<float>(S.c02, ex, ey, ez), __ldg(S.y[4] + i));
  const c32 c12 = cscale(shift_phase<float>(S.c12, ex, ey, ez), __ldg(S.y[5] + i));
  const float d00 = __ldg(S.y[0] + i), d11 = __ldg(S.y[1] + i), d22 = __ldg(S.y[2] + i);
  const c32 b0 = cscale(a0, d00) + c01 * a1 + c02 * a2;
  const c32 b1 = cmulc(a0, c01) + cscale(a1, d11) + c12 * a2;
  const c32 b2 = cmulc(a0, c02) + cmulc(a1, c12) + cscale(a2, d22);
  a0 = b0;
  a1 = b1;
  a2 = b2;
}

// forward first group from the staged rows (row < nz; zero beyond) into the tile
template <int Q>
__device__ __forceinline__ void stg_first_fwd(const c32* stg, int nz, c32* buf, const AxPlan& p,
                                              const c32* W) {
  constexpr int N = 1 << Q;
  const int lh = p.n - Q;
  const int tasks = TX << lh;
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int k = t >> LTX;
    c32 v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) {
      const int row = k + (r << lh);
      v[r] = row < nz ? stg[(row << LTX) + col] : mk<float>(0, 0);
    }
    dft_dif<float, Q>(v);
    group_twiddle<float, Q, false>(v, k, 0, W);
#pragma unroll
    for (int r = 0; r < N; ++r) buf[((k + (r << lh)) << LTX) + col] = v[r];
  }
}

// fused middle step of the three face families with the y/z-folded spectra
template <int Q>
__device__ __forceinline__ void z3_fused_yz(c32* buf, size_t tsz, const AxPlan& p,
                                            const PSpec& S, const YzIdx& Y, int kx0,
                                            const c32& ey) {
  constexpr int N = 1 << Q;
  const int tasks = TX << (p.n - Q);
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int start = (t >> LTX) << Q;
    c32 v[3][N];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
#pragma unroll
      for (int r = 0; r < N; ++r) v[f][r] = buf[f * tsz + ((start + r) << LTX) + col];
      dft_dif<float, Q>(v[f]);
    }
    const c32 ex = S.ex32[kx0 + col];
#pragma unroll
    for (int r = 0; r < N; ++r) pspec_apply_yz(S, Y, col, start + r, ex, ey, v[0][r], v[1][r], v[2][r]);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      dft_dit<float, Q>(v[f]);
#pragma unroll
      for (int r = 0; r < N; ++r) buf[f * tsz + ((start + r) << LTX) + col] = v[f][r];
    }
  }
}

// fused middle step of one edge family (real y/z-folded spectrum)
template <int Q>
__device__ __forceinline__ void z1_fused_yz(c32* buf, const AxPlan& p, const float* __restrict__ sy,
                                            const YzIdx& Y) {
  constexpr int N = 1 << Q;
  const int tasks = TX << (p.n - Q);
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & (TX - 1);
    const int start = (t >> LTX) << Q;
    c32 v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = buf[((start + r) << LTX) + col];
    dft_dif<float, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = cscale(v[r], __ldg(sy + Y.at(col, start + r)));
    dft_dit<float, Q>(v);
#pragma unroll
    for (int r = 0; r < N; ++r) buf[((start + r) << LTX) + col] = v[r];
  }
}

// One family's pencil rows of a tile, for the staging warp.
struct StageSrc {
  const c32* T;  // family buffer at the tile's (ky, kx0)
  int nz;        // occupied z rows
};

// the staging warp (warp 0): arm the barrier with the tile's bytes, then one bulk copy
// per staged row, lanes striding over the rows
__device__ __forceinline__ void stage_tile(uint64_t* bar, c32* stg, int nzs, const StageSrc* src,
                                           int nfam, size_t pl) {
  const int lane = threadIdx.x & 31;
  uint32_t bytes = 0;
  for (int f = 0; f < nfam; ++f) bytes += (uint32_t)src[f].nz * (TX * sizeof(c32));
  if (lane == 0) mbar_arrive_expect_tx(bar, bytes);
  __syncwarp();
  for (int f = 0; f < nfam; ++f)
    for (int z = lane; z < src[f].nz; z += 32)
      bulk_g2s(stg + ((size_t)f * nzs + z) * TX, src[f].T + (size_t)z * pl, TX * sizeof(c32), bar);
}

// every thread waits for the staged tile; false (for all threads alike) if any wait ran
// into its limit, after the copies in flight were waited for once more
__device__ __forceinline__ bool stage_wait(uint64_t* bar, uint32_t parity, int* err) {
  const bool ok = mbar_wait_bounded(bar, parity, ZWAIT_LIMIT);
  if (__syncthreads_and(ok)) return true;
  if (threadIdx.x == 0) atomicExch(err, 1);
  mbar_wait_bounded(bar, parity, ZWAIT_LIMIT);
  return false;
}

template <int Q0, int QL>
__global__ void __launch_bounds__(ZTPB, 3) k_zconv3_staged(c32* T0, c32* T1, c32* T2, int nz0,
                                                           int nz1, int nz2, int nzs, PSpec S,
                                                           int Lx, int Ly, AxPlan p,
                                                           const c32* __restrict__ twm,
                                                           int twmax, int ntiles, int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int Lz = 1 << p.n;
  const size_t tsz = (size_t)Lz << LTX;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  c32* W = reinterpret_cast<c32*>(smem_raw + 128);
  c32* buf = W + Lz;             // three work tiles, family f at buf + f*tsz
  c32* stg = buf + 3 * tsz;      // staged rows, family f at stg + f*nzs*TX
  const int ntx = Lx >> LTX;
  const size_t pl = (size_t)Ly * Lx;
  c32* Tf[3] = {T0, T1, T2};
  const int nzf[3] = {nz0, nz1, nz2};
  auto sources = [&](int tile, StageSrc* src) {
    const size_t off = (size_t)(tile / ntx) * Lx + ((tile % ntx) << LTX);
    for (int f = 0; f < 3; ++f) src[f] = StageSrc{Tf[f] + off, nzf[f]};
  };
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  int tile = blockIdx.x;
  if (threadIdx.x < 32 && tile < ntiles) {
    StageSrc src[3];
    sources(tile, src);
    stage_tile(bar, stg, nzs, src, 3, pl);
  }
  load_twiddles<float>(W, twm, twmax, Lz);
  __syncthreads();
  uint32_t parity = 0;
  for (; tile < ntiles; tile += gridDim.x) {
    const int ky = tile / ntx, kx0 = (tile % ntx) << LTX;
    if (!stage_wait(bar, parity, err)) return;
    parity ^= 1u;
    qpick<Q0, QCap<float>::XY>(p.q[0], [&](auto QC) {
      stg_first_fwd<decltype(QC)::value>(stg, nz0, buf, p, W);
      stg_first_fwd<decltype(QC)::value>(stg + (size_t)nzs * TX, nz1, buf + tsz, p, W);
      stg_first_fwd<decltype(QC)::value>(stg + 2 * (size_t)nzs * TX, nz2, buf + 2 * tsz, p, W);
    });
    __syncthreads();
    // the stage is free: fetch the next tile while this one computes
    const int next = tile + gridDim.x;
    if (threadIdx.x < 32 && next < ntiles) {
      fence_proxy_async_smem();
      StageSrc src[3];
      sources(next, src);
      stage_tile(bar, stg, nzs, src, 3, pl);
    }
    {
      int s = p.q[0];
      for (int g = 1; g + 1 < p.ng; ++g) {
        smem_group_q<float, false, LTX>(buf, TX, p.q[g], p.n, s, W);
        smem_group_q<float, false, LTX>(buf + tsz, TX, p.q[g], p.n, s, W);
        smem_group_q<float, false, LTX>(buf + 2 * tsz, TX, p.q[g], p.n, s, W);
        s += p.q[g];
        __syncthreads();
      }
    }
    const YzIdx Y = make_yzidx(Lx, Ly, Lz, kx0, ky);
    const c32 ey = S.ey32[ky];
    qpick<QL, QCap<float>::Z3>(p.q[p.ng - 1], [&](auto QC) {
      z3_fused_yz<decltype(QC)::value>(buf, tsz, p, S, Y, kx0, ey);
    });
    __syncthreads();
    {
      int s = p.n - p.q[p.ng - 1];
      for (int g = p.ng - 2; g >= 1; --g) {
        s -= p.q[g];
        smem_group_q<float, true, LTX>(buf, TX, p.q[g], p.n, s, W);
        smem_group_q<float, true, LTX>(buf + tsz, TX, p.q[g], p.n, s, W);
        smem_group_q<float, true, LTX>(buf + 2 * tsz, TX, p.q[g], p.n, s, W);
        __syncthreads();
      }
    }
    const size_t off = (size_t)ky * Lx + kx0;
    qpick<Q0, QCap<float>::XY>(p.q[0], [&](auto QC) {
      col_last_inv<float, decltype(QC)::value>(buf, T0 + off, pl, TX, nz0, p, W);
      col_last_inv<float, decltype(QC)::value>(buf + tsz, T1 + off, pl, TX, nz1, p, W);
      col_last_inv<float, decltype(QC)::value>(buf + 2 * tsz, T2 + off, pl, TX, nz2, p, W);
    });
    __syncthreads();  // the work tiles are rewritten by the next tile's first group
  }
}

// the edge families' z passes in one launch; all share one circulant grid (Lx, Ly, Lz)
struct EdgeSet {
  c32* T[3];
  int nz[3];
  const float* sy[3];
  int nf;
};

template <int Q0, int QL>
__global__ void __launch_bounds__(ZTPB, 4) k_zedge_staged(EdgeSet E, int nzs, int Lx, int Ly,
                                                          AxPlan p, const c32* __restrict__ twm,
                                                          int twmax, int tiles_per_fam,
                                                          int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int Lz = 1 << p.n;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  c32* W = reinterpret_cast<c32*>(smem_raw + 128);
  c32* buf = W + Lz;
  c32* stg = buf + ((size_t)Lz << LTX);
  const int ntx = Lx >> LTX;
  const size_t pl = (size_t)Ly * Lx;
  const int ntiles = tiles_per_fam * E.nf;
  auto source = [&](int tile, StageSrc* src) {
    const int f = tile / tiles_per_fam, t = tile - f * tiles_per_fam;
    const size_t off = (size_t)(t / ntx) * Lx + ((t % ntx) << LTX);
    src[0] = StageSrc{E.T[f] + off, E.nz[f]};
  };
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  int tile = blockIdx.x;
  if (threadIdx.x < 32 && tile < ntiles) {
    StageSrc src[1];
    source(tile, src);
    stage_tile(bar, stg, nzs, src, 1, pl);
  }
  load_twiddles<float>(W, twm, twmax, Lz);
  __syncthreads();
  uint32_t parity = 0;
  for (; tile < ntiles; tile += gridDim.x) {
    const int f = tile / tiles_per_fam, t = tile - f * tiles_per_fam;
    const int ky = t / ntx, kx0 = (t % ntx) << LTX;
    const int nz = E.nz[f];
    if (!stage_wait(bar, parity, err)) return;
    parity ^= 1u;
    qpick<Q0, QCap<float>::XY>(p.q[0], [&](auto QC) {
      stg_first_fwd<decltype(QC)::value>(stg, nz, buf, p, W);
    });
    __syncthreads();
    const int next = tile + gridDim.x;
    if (threadIdx.x < 32 && next < ntiles) {
      fence_proxy_async_smem();
      StageSrc src[1];
      source(next, src);
      stage_tile(bar, stg, nzs, src, 1, pl);
    }
    middle_groups<float, false, LTX>(buf, TX, p, W);
    const YzIdx Y = make_yzidx(Lx, Ly, Lz, kx0, ky);
    qpick<QL, QCap<float>::Z1>(p.q[p.ng - 1], [&](auto QC) {
      z1_fused_yz<decltype(QC)::value>(buf, p, E.sy[f], Y);
    });
    __syncthreads();
    middle_groups<float, true, LTX>(buf, TX, p, W);
    const size_t off = (size_t)ky * Lx + kx0;
    qpick<Q0, QCap<float>::XY>(p.q[0], [&](auto QC) {
      col_last_inv<float, decltype(QC)::value>(buf, E.T[f] + off, pl, TX, nz, p, W);
    });
    __syncthreads();
  }
}

// Register-direct FP32 z passes on the y/z-folded spectra (ZTune form 1): k_zconv3 /
// k_zconv1 with the spectral step of the staged kernels; whole 16-column tiles.
template <int Q0, int QL>
__global__ void __launch_bounds__(ZTPB, 4) k_zconv3_yz(c32* T0, c32* T1, c32* T2, int nz0,
                                                       int nz1, int nz2, PSpec S, int Lx, int Ly,
                                                       AxPlan p, const c32* __restrict__ twm,
                                                       int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int Lz = 1 << p.n;
  const size_t tsz = (size_t)Lz << LTX;
  c32* W = reinterpret_cast<c32*>(smem_raw);
  c32* buf = W + Lz;
  const int kx0 = blockIdx.x * TX, ky = blockIdx.y;
  const size_t pl = (size_t)Ly * Lx;
  const size_t off = (size_t)ky * Lx + kx0;
  T0 += off;
  T1 += off;
  T2 += off;
  load_twiddles<float>(W, twm, twmax, Lz);
  __syncthreads();
  qpick<Q0, QCap<float>::XY>(p.q[0], [&](auto QC) {
    col_first_fwd<float, decltype(QC)::value>(T0, pl, TX, nz0, buf, p, W, T0);
    col_first_fwd<float, decltype(QC)::value>(T1, pl, TX, nz1, buf + tsz, p, W, T1);
    col_first_fwd<float, decltype(QC)::value>(T2, pl, TX, nz2, buf + 2 * tsz, p, W, T2);
  });
  __syncthreads();
  {
    int s = p.q[0];
    for (int g = 1; g + 1 < p.ng; ++g) {
      smem_group_q<float, false, LTX>(buf, TX, p.q[g], p.n, s, W);
      smem_group_q<float, false, LTX>(buf + tsz, TX, p.q[g], p.n, s, W);
      smem_group_q<float, false, LTX>(buf + 2 * tsz, TX, p.q[g], p.n, s, W);
      s += p.q[g];
      __syncthreads();
    }
  }
  const YzIdx Y = make_yzidx(Lx, Ly, Lz, kx0, ky);
  const c32 ey = S.ey32[ky];
  qpick<QL, QCap<float>::Z3>(p.q[p.ng - 1], [&](auto QC) {
    z3_fused_yz<decltype(QC)::value>(buf, tsz, p, S, Y, kx0, ey);
  });
  __syncthreads();
  {
    int s = p.n - p.q[p.ng - 1];
    for (int g = p.ng - 2; g >= 1; --g) {
      s -= p.q[g];
      smem_group_q<float, true, LTX>(buf, TX, p.q[g], p.n, s, W);
      smem_group_q<float, true, LTX>(buf + tsz, TX, p.q[g], p.n, s, W);
      smem_group_q<float, true, LTX>(buf + 2 * tsz, TX, p.q[g], p.n, s, W);
      __syncthreads();
    }
  }
  qpick<Q0, QCap<float>::XY>(p.q[0], [&](auto QC) {
    col_last_inv<float, decltype(QC)::value>(buf, T0, pl, TX, nz0, p, W);
    col_last_inv<float, decltype(QC)::value>(buf + tsz, T1, pl, TX, nz1, p, W);
    col_last_inv<float, decltype(QC)::value>(buf + 2 * tsz, T2, pl, TX, nz2, p, W);
  });
}

template <int Q0, int QL>
__global__ void __launch_bounds__(ZTPB, 4) k_zconv1_yz(c32* T0, int nz0, const float* __restrict__ sy,
                                                       int Lx, int Ly, AxPlan p,
                                                       const c32* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int Lz = 1 << p.n;
  c32* W = reinterpret_cast<c32*>(smem_raw);
  c32* buf = W + Lz;
  const int kx0 = blockIdx.x * TX, ky = blockIdx.y;
  const size_t pl = (size_t)Ly * Lx;
  c32* Tg = T0 + (size_t)ky * Lx + kx0;
  load_twiddles<float>(W, twm, twmax, Lz);
  __syncthreads();
  qpick<Q0, QCap<float>::XY>(p.q[0], [&](auto QC) {
    col_first_fwd<float, decltype(QC)::value>(Tg, pl, TX, nz0, buf, p, W, Tg);
  });
  __syncthreads();
  middle_groups<float, false, LTX>(buf, TX, p, W);
  const YzIdx Y = make_yzidx(Lx, Ly, Lz, kx0, ky);
  qpick<QL, QCap<float>::Z1>(p.q[p.ng - 1], [&](auto QC) {
    z1_fused_yz<decltype(QC)::value>(buf, p, sy, Y);
  });
  __syncthreads();
  middle_groups<float, true, LTX>(buf, TX, p, W);
  qpick<Q0, QCap<float>::XY>(p.q[0], [&](auto QC) {
    col_last_inv<float, decltype(QC)::value>(buf, Tg, pl, TX, nz0, p, W);
  });
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
    set_error("shared memory tile exceeds 227 KB: z extent too large for the z-pass tiles");
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
  static AxPlan z3(int n) {
    return QCap<R>::wide ? make_plan(n, 2, 4, 2) : make_plan(n, 3, 4, 3);
  }
  // alt (FP32 only): the alternative edge plan the tuner may pick (first group 16 points)
  static AxPlan z1(int n, int alt = 0) {
    if (QCap<R>::wide) return make_plan(n, 3, 4, 3);
    return alt ? make_plan(n, 4, 4, 3) : make_plan(n, 4, 4, 4);
  }
};

template <typename R>
struct Launch {
  static cx<R>* buf(const Family& f) { return reinterpret_cast<cx<R>*>(f.T[slot_of<R>()]); }
  // kind 0: forward x, 1: inverse x, 2: forward y, 3: inverse y; io[f]: the compact
  // vector of family f (x passes)
  static int pass(int kind, const Family* F, int nfam, c64* const* io, const cx<R>* tw,
                  int twmax, cudaStream_t st) {
    PassSet<R> s{};
    int ctas = 0;
    size_t sm = 0;
    for (int f = 0; f < nfam; ++f) {
      if (!F[f].active) continue;
      if (s.nf == kMaxFam) return set_error("too many families in one pass"), PEEC_ERR_UNSUPPORTED_INTERNAL;
      const Family& fam = F[f];
      FamPass<R>& d = s.f[s.nf++];
      d.T = buf(fam);
      d.map = fam.map;
      d.io = io ? io[f] : nullptr;
      d.cta0 = ctas;
      int gy = fam.dims[2];
      if (kind < 2) {
        const int Lx = fam.L[0];
        d.p = Plans<R>::xy(fam.logL[0]);
        d.L_other = fam.L[1];
        d.a = fam.dims[0];
        d.b = fam.dims[1];
        d.gx = (fam.dims[1] + TY - 1) / TY;
        sm = std::max(sm, sizeof(cx<R>) * (Lx + (size_t)Lx * XRS));
      } else {
        const int Ly = fam.L[1];
        d.p = Plans<R>::xy(fam.logL[1]);
        d.L_other = fam.L[0];
        d.a = kind == 3 ? Ly : fam.dims[1];
        d.b = kind == 3 ? fam.dims[1] : Ly;
        d.gx = (fam.L[0] + TX - 1) / TX;
        sm = std::max(sm, sizeof(cx<R>) * (Ly + ((size_t)Ly << LTX)));
      }
      ctas += d.gx * gy;
    }
    if (s.nf == 0) return 0;
    switch (kind) {
      case 0:
        CTX_CHECK(smem_optin(k_xfwd<R>, sm));
        k_xfwd<R><<<ctas, TPB, sm, st>>>(s, tw, twmax);
        break;
      case 1:
        CTX_CHECK(smem_optin(k_xinv<R>, sm));
        k_xinv<R><<<ctas, TPB, sm, st>>>(s, tw, twmax);
        break;
      case 2:
        CTX_CHECK(smem_optin(k_ypass<R, false>, sm));
        k_ypass<R, false><<<ctas, TPB, sm, st>>>(s, tw, twmax);
        break;
      default:
        CTX_CHECK(smem_optin(k_ypass<R, true>, sm));
        k_ypass<R, true><<<ctas, TPB, sm, st>>>(s, tw, twmax);
        break;
    }
    return 0;
  }
  static int zconv3(const Family* F, const PSpec& S, const cx<R>* tw, int twmax,
                    cudaStream_t st) {
    const int Lz = F[0].L[2];
    const size_t sm = sizeof(cx<R>) * (Lz + 3 * ((size_t)Lz << LTX));
    const AxPlan p = Plans<R>::z3(F[0].logL[2]);
    constexpr int QL = QCap<R>::Z3;
    const bool spec = p.ng >= 2 && p.q[0] == 4 && p.q[p.ng - 1] == QL;
    auto kern = spec ? k_zconv3<R, 4, QL> : k_zconv3<R, 0, 0>;
    CTX_CHECK(smem_optin(kern, sm));
    dim3 g((F[0].L[0] + TX - 1) / TX, F[0].L[1]);
    kern<<<g, ZTPB, sm, st>>>(buf(F[0]), buf(F[1]), buf(F[2]), F[0].dims[2], F[1].dims[2],
                              F[2].dims[2], S, F[0].L[0], F[0].L[1], p, tw, twmax);
    return 0;
  }
  static int zconv1(const Family& f, const void* s, const cx<R>* tw, int twmax, cudaStream_t st,
                    int alt = 0) {
    const int Lz = f.L[2];
    const size_t sm = sizeof(cx<R>) * (Lz + ((size_t)Lz << LTX));
    const AxPlan p = Plans<R>::z1(f.logL[2], alt);
    constexpr int QL = QCap<R>::Z1;
    const int q0 = p.q[0], ql = p.q[p.ng - 1];
    auto kern = (p.ng >= 2 && q0 == 4 && ql == QL) ? k_zconv1<R, 4, QL>
                : (p.ng >= 2 && q0 == 4 && ql == 3)  ? k_zconv1<R, 4, 3>
                : (p.ng >= 2 && q0 == 3 && ql == QL) ? k_zconv1<R, 3, QL>
                                                     : k_zconv1<R, 0, 0>;
    CTX_CHECK(smem_optin(kern, sm));
    dim3 g((f.L[0] + TX - 1) / TX, f.L[1]);
    kern<<<g, ZTPB, sm, st>>>(buf(f), f.dims[2], s, f.L[0], f.L[1], p, tw, twmax);
    return 0;
  }
};

// The FP32 z-pass forms (ZTune): direct on full-form spectra, direct on y/z-folded
// spectra, staged. Templates, so that only the float instantiation compiles their kernels.
template <typename R>
static PSpec pspec_of(const Spectrum* spec, const void* const* ph) {
  const int p = slot_of<R>();
  PSpec S{spec[0].d[p], spec[1].d[p], spec[2].d[p], spec[3].d[p], spec[4].d[p], spec[5].d[p],
          spec[0].oct,  spec[1].oct,  spec[2].oct,  spec[3].oct,  spec[4].oct,  spec[5].oct,
          ph[0],        ph[1],        ph[2],        {},           {},           {}};
  for (int a = 0; a < 3; ++a) {
    S.c01[a] = spec[3].c[a];
    S.c02[a] = spec[4].c[a];
    S.c12[a] = spec[5].c[a];
  }
  if (std::is_same<R, float>::value) {
    for (int i = 0; i < 6; ++i) S.y[i] = (const float*)spec[i].yz32;
    S.ex32 = (const c32*)ph[3];
    S.ey32 = (const c32*)ph[4];
    S.ez32 = (const c32*)ph[5];
  }
  return S;
}

template <int UNUSED = 0>
static int zface_f32(const Family* F, int nfam, const PSpec& S, const c32* tw, int twmax,
                     const ZTune& zt, cudaStream_t st) {
  const int form = zpass_yz_faces(F, nfam) ? zt.face : 0;
  if (form == 0) return Launch<float>::zconv3(F, S, tw, twmax, st);
  const int Lz = F[0].L[2], Lx = F[0].L[0], Ly = F[0].L[1];
  const AxPlan p = Plans<float>::z3(F[0].logL[2]);
  constexpr int QL = QCap<float>::Z3;
  const bool spec = p.q[0] == 4 && p.q[p.ng - 1] == QL;
  c32* T0 = Launch<float>::buf(F[0]);
  c32* T1 = Launch<float>::buf(F[1]);
  c32* T2 = Launch<float>::buf(F[2]);
  if (form == 1) {
    const size_t sm = sizeof(c32) * (Lz + 3 * ((size_t)Lz << LTX));
    auto kern = spec ? k_zconv3_yz<4, QL> : k_zconv3_yz<0, 0>;
    CTX_CHECK(smem_optin(kern, sm));
    dim3 g(Lx >> LTX, Ly);
    kern<<<g, ZTPB, sm, st>>>(T0, T1, T2, F[0].dims[2], F[1].dims[2], F[2].dims[2], S, Lx, Ly,
                              p, tw, twmax);
    return 0;
  }
  const int nzs = std::max(F[0].dims[2], std::max(F[1].dims[2], F[2].dims[2]));
  const size_t sm = 128 + sizeof(c32) * (Lz + 3 * ((size_t)Lz << LTX) + 3 * (size_t)nzs * TX);
  auto kern = spec ? k_zconv3_staged<4, QL> : k_zconv3_staged<0, 0>;
  CTX_CHECK(smem_optin(kern, sm));
  const int ntiles = (Lx >> LTX) * Ly;
  const int per_sm = std::max(1, std::min(3, (int)((227 * 1024) / (sm + 1024))));
  const int grid = std::min(ntiles, zt.nsm * per_sm);
  kern<<<grid, ZTPB, sm, st>>>(T0, T1, T2, F[0].dims[2], F[1].dims[2], F[2].dims[2], nzs, S,
                               Lx, Ly, p, tw, twmax, ntiles, zt.err);
  return 0;
}

template <int UNUSED = 0>
static int zedge_f32(const Family* F, int nfam, const Spectrum* spec, const c32* tw, int twmax,
                     const ZTune& zt, cudaStream_t st) {
  const int form = zpass_yz_edges(F, nfam) ? zt.edge : 0;
  if (form < 2) {
    for (int f = 3; f < nfam; ++f) {
      if (!F[f].active) continue;
      if (form == 0) {
        CTX_CHECK(Launch<float>::zconv1(F[f], spec[3 + f].d[1], tw, twmax, st, zt.edge_plan));
        continue;
      }
      const Family& fam = F[f];
      const int Lz = fam.L[2];
      const AxPlan p = Plans<float>::z1(fam.logL[2], zt.edge_plan);
      const int q0 = p.q[0], ql = p.q[p.ng - 1];
      auto kern = (q0 == 4 && ql == 3) ? k_zconv1_yz<4, 3>
                  : (q0 == 3 && ql == 4) ? k_zconv1_yz<3, 4>
                                         : k_zconv1_yz<0, 0>;
      const size_t sm = sizeof(c32) * (Lz + ((size_t)Lz << LTX));
      CTX_CHECK(smem_optin(kern, sm));
      dim3 g(fam.L[0] >> LTX, fam.L[1]);
      kern<<<g, ZTPB, sm, st>>>(Launch<float>::buf(fam), fam.dims[2],
                                (const float*)spec[3 + f].yz32, fam.L[0], fam.L[1], p, tw,
                                twmax);
    }
    return 0;
  }
  EdgeSet E{};
  const Family* f0 = nullptr;
  int nzs = 0;
  for (int f = 3; f < nfam; ++f) {
    if (!F[f].active) continue;
    if (!f0) f0 = &F[f];
    E.T[E.nf] = Launch<float>::buf(F[f]);
    E.nz[E.nf] = F[f].dims[2];
    E.sy[E.nf] = (const float*)spec[3 + f].yz32;
    nzs = std::max(nzs, F[f].dims[2]);
    ++E.nf;
  }
  if (!f0) return 0;
  const int Lz = f0->L[2], Lx = f0->L[0], Ly = f0->L[1];
  const AxPlan p = Plans<float>::z1(f0->logL[2], zt.edge_plan);
  const size_t sm = 128 + sizeof(c32) * (Lz + ((size_t)Lz << LTX) + (size_t)nzs * TX);
  const int q0 = p.q[0], ql = p.q[p.ng - 1];
  auto kern = (q0 == 4 && ql == 3) ? k_zedge_staged<4, 3>
              : (q0 == 3 && ql == 4) ? k_zedge_staged<3, 4>
                                     : k_zedge_staged<0, 0>;
  CTX_CHECK(smem_optin(kern, sm));
  const int per_fam = (Lx >> LTX) * Ly;
  const int per_sm = std::max(1, std::min(4, (int)((227 * 1024) / (sm + 1024))));
  const int grid = std::min(per_fam * E.nf, zt.nsm * per_sm);
  kern<<<grid, ZTPB, sm, st>>>(E, nzs, Lx, Ly, p, tw, twmax, per_fam, zt.err);
  return 0;
}

// ev (nullable): 6 events bracketing the five pass classes
// ph: the face grid's phase tables (x, y, z), complex FP64, then complex FP32
// zt (nullable): the FP32 z-pass forms (form 0 when null)
template <typename R>
int conv_all_t(const Family* F, int nfam, const Spectrum* spec, const void* const* ph,
               const c64* x, c64* LpI, c64* PQ, int64_t m, const cx<R>* tw, int twmax,
               cudaStream_t st, cudaEvent_t* ev, const ZTune* zt) {
  using Lc = Launch<R>;
  const int p = slot_of<R>();
  if (nfam > kMaxFam) return set_error("too many families"), PEEC_ERR_UNSUPPORTED_INTERNAL;
  c64* in[kMaxFam];
  c64* out[kMaxFam];
  for (int f = 0; f < nfam; ++f) {
    in[f] = const_cast<c64*>(F[f].lp ? x : x + m);
    out[f] = F[f].lp ? LpI : PQ;
  }
  if (ev) cudaEventRecord(ev[0], st);
  CTX_CHECK(Lc::pass(0, F, nfam, in, tw, twmax, st));
  if (ev) cudaEventRecord(ev[1], st);
  CTX_CHECK(Lc::pass(2, F, nfam, nullptr, tw, twmax, st));
  if (ev) cudaEventRecord(ev[2], st);
  const PSpec S = pspec_of<R>(spec, ph);
  if constexpr (std::is_same<R, float>::value) {
    const ZTune z0{};
    const ZTune& z = zt ? *zt : z0;
    CTX_CHECK(zface_f32(F, nfam, S, tw, twmax, z, st));
    CTX_CHECK(zedge_f32(F, nfam, spec, tw, twmax, z, st));
  } else {
    CTX_CHECK(Lc::zconv3(F, S, tw, twmax, st));
    for (int f = 3; f < nfam; ++f)
      if (F[f].active)
        CTX_CHECK(Lc::zconv1(F[f], octant_spectra<R>() ? spec[3 + f].oct : spec[3 + f].d[p], tw,
                             twmax, st));
  }
  if (ev) cudaEventRecord(ev[3], st);
  CTX_CHECK(Lc::pass(3, F, nfam, nullptr, tw, twmax, st));
  if (ev) cudaEventRecord(ev[4], st);
  CTX_CHECK(Lc::pass(1, F, nfam, out, tw, twmax, st));
  if (ev) cudaEventRecord(ev[5], st);
  return 0;
}

}  // namespace peec
