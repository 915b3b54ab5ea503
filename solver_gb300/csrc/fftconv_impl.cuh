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
  static AxPlan z1(int n) {
    return QCap<R>::wide ? make_plan(n, 3, 4, 3) : make_plan(n, 4, 4, 4);
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
  static int zconv1(const Family& f, const void* s, const cx<R>* tw, int twmax, cudaStream_t st) {
    const int Lz = f.L[2];
    const size_t sm = sizeof(cx<R>) * (Lz + ((size_t)Lz << LTX));
    const AxPlan p = Plans<R>::z1(f.logL[2]);
    constexpr int QL = QCap<R>::Z1;
    const bool spec = p.ng >= 2 && p.q[0] == 4 && p.q[p.ng - 1] == QL;
    auto kern = spec ? k_zconv1<R, 4, QL> : k_zconv1<R, 0, 0>;
    CTX_CHECK(smem_optin(kern, sm));
    dim3 g((f.L[0] + TX - 1) / TX, f.L[1]);
    kern<<<g, ZTPB, sm, st>>>(buf(f), f.dims[2], s, f.L[0], f.L[1], p, tw, twmax);
    return 0;
  }
};

// ev (nullable): 6 events bracketing the five pass classes
// ph: the face grid's phase tables (x, y, z), complex FP64
template <typename R>
int conv_all_t(const Family* F, int nfam, const Spectrum* spec, const void* const* ph,
               const c64* x, c64* LpI, c64* PQ, int64_t m, const cx<R>* tw, int twmax,
               cudaStream_t st, cudaEvent_t* ev) {
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
  PSpec S{spec[0].d[p], spec[1].d[p], spec[2].d[p], spec[3].d[p], spec[4].d[p], spec[5].d[p],
          spec[0].oct,  spec[1].oct,  spec[2].oct,  spec[3].oct,  spec[4].oct,  spec[5].oct,
          ph[0],        ph[1],        ph[2],        {},           {},           {}};
  for (int a = 0; a < 3; ++a) {
    S.c01[a] = spec[3].c[a];
    S.c02[a] = spec[4].c[a];
    S.c12[a] = spec[5].c[a];
  }
  CTX_CHECK(Lc::zconv3(F, S, tw, twmax, st));
  for (int f = 3; f < nfam; ++f)
    if (F[f].active)
      CTX_CHECK(Lc::zconv1(F[f], octant_spectra<R>() ? spec[3 + f].oct : spec[3 + f].d[p], tw,
                           twmax, st));
  if (ev) cudaEventRecord(ev[3], st);
  CTX_CHECK(Lc::pass(3, F, nfam, nullptr, tw, twmax, st));
  if (ev) cudaEventRecord(ev[4], st);
  CTX_CHECK(Lc::pass(1, F, nfam, out, tw, twmax, st));
  if (ev) cudaEventRecord(ev[5], st);
  return 0;
}

}  // namespace peec
