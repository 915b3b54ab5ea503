// Vector kernels of the Householder GMRES (compact-WY form).
//
// The reflector basis U (N x kmax, column-major, complex double) is applied with
// two passes per application instead of the reference's one dot+axpy per
// reflector (gmres_custom.jl:112-127): a multi-dot z = U(:,0:k)^H v, a small
// triangular product on the host, and a multi-axpy v -= U(:,0:k) c. Reductions
// are deterministic: warp-shuffle partials per CTA, then a fixed-order sum.
#include <mutex>

#include "ctx.hpp"
#include "peec_gb300.h"

namespace peec {

// Basis storage: complex double (the FP64 solves) or complex float-float (the inner
// solves of the mixed solve), and the arithmetic follows the storage. GB300 runs FP64 at
// about 1/60 of its FP32 rate, and these kernels do eight flops per basis element and
// column, so with FP64 arithmetic they are FP64-pipe bound at a fraction of HBM speed;
// float-float arithmetic (FP32 error-free transformations, ~2^-48) keeps the basis at
// FP64-like accuracy with the same 16 bytes per element and runs at HBM speed.
template <typename T>
struct BasisArith;
template <>
struct BasisArith<c64> {
  using A = double;
};
template <>
struct BasisArith<cff> {
  using A = ff;
};
template <typename A, typename T>
__device__ __forceinline__ cx<A> as(const T& v) {
  return mk<A>((A)v.x, (A)v.y);
}

constexpr int KB = 8;        // columns per multi-dot tile
constexpr int RED_TPB = 256;
constexpr int MD_BLOCKS_MAX = 152 * 2;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// partial[c0+c][blk] (complex) = sum over the CTA's rows of conj(U[i,c0+c]) * v[i],
// c < NC: the tile's columns are a template parameter, so loads, products and the
// shuffle reductions are exactly the ones needed; each thread walks at least eight rows
// DYN: the column count and the vector come from the device loop's iteration index
// (k = *dj + koff, v += *dj * vstep); column tiles past k leave at once, the last tile
// masks its columns. Per column the arithmetic and the summation order are those of the
// fixed-count form.
template <int NC, typename UT, typename VT, bool DYN = false>
__global__ void __launch_bounds__(RED_TPB) k_multidot(const UT* __restrict__ U, size_t ldu,
                                                      const VT* __restrict__ v, size_t N,
                                                      int c0, c64* partial,
                                                      const int* __restrict__ dj = nullptr,
                                                      int koff = 0, size_t vstep = 0) {
  using A = typename BasisArith<UT>::A;
  __shared__ double red[RED_TPB / 32][2 * NC];
  c0 += blockIdx.y * NC;
  int nc = NC;
  if (DYN) {
    const int jj = *dj;
    v += (size_t)jj * vstep;
    nc = jj + koff - c0;
    if (nc <= 0) return;  // the whole CTA: no barrier has been reached
    if (nc > NC) nc = NC;
  }
  const UT* __restrict__ Uc = U + (size_t)c0 * ldu;
  A ar[NC], ai[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) ar[c] = ai[c] = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) {
    cx<A> u[NC];
    const cx<A> x = as<A>(v[i]);
#pragma unroll
    for (int c = 0; c < NC; ++c)
      if (!DYN || c < nc) u[c] = as<A>(Uc[(size_t)c * ldu + i]);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (!DYN || c < nc) {
        ar[c] = ar[c] + (u[c].x * x.x + u[c].y * x.y);
        ai[c] = ai[c] + (u[c].x * x.y - u[c].y * x.x);
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const double sr = warp_sum((double)ar[c]), si = warp_sum((double)ai[c]);
    if (lane == 0) {
      red[wid][2 * c] = sr;
      red[wid][2 * c + 1] = si;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * nc) {
    double s = 0.0;
    for (int w = 0; w < RED_TPB / 32; ++w) s += red[w][threadIdx.x];
    const int c = threadIdx.x >> 1;
    double* p = reinterpret_cast<double*>(partial + (size_t)(c0 + c) * gridDim.x + blockIdx.x);
    p[threadIdx.x & 1] = s;
  }
}

// out[c] = sum_b partial[c][b]: one warp per column, lane-strided then a shuffle tree
// (fixed order for a fixed block count)
__global__ void k_reduce_cols(const c64* __restrict__ partial, int nblk, int k, c64* out,
                              const int* __restrict__ dj = nullptr) {
  if (dj) k += *dj;  // device loop: k is an offset from the iteration index
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= k) return;  // whole warps leave together
  double sr = 0.0, si = 0.0;
  for (int b = lane; b < nblk; b += 32) {
    const c64 p = partial[(size_t)c * nblk + b];
    sr += p.x;
    si += p.y;
  }
  sr = warp_sum(sr);
  si = warp_sum(si);
  if (lane == 0) out[c] = mk<double>(sr, si);
}

// v[i] = base[i] (or e_unit) - sum_c U[i,c]*coef[c];  optional tail |v|^2 partials for i >= tail0
template <typename UT>
__global__ void __launch_bounds__(RED_TPB) k_multiaxpy(const UT* __restrict__ U, size_t ldu,
                                                       const c64* __restrict__ base, int unit,
                                                       const c64* __restrict__ coef, int k,
                                                       size_t N, c64* out, size_t tail0,
                                                       double* tailpart,
                                                       const int* __restrict__ dj = nullptr) {
  using A = typename BasisArith<UT>::A;
  if (dj) {  // device loop: k, unit and tail0 are offsets from the iteration index
    const int jj = *dj;
    k += jj;
    unit += jj;
    tail0 += (size_t)jj;
  }
  extern __shared__ unsigned char sc_raw[];
  cx<A>* sc = reinterpret_cast<cx<A>*>(sc_raw);
  for (int c = threadIdx.x; c < k; c += blockDim.x) sc[c] = as<A>(coef[c]);
  __syncthreads();
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    c64 x;
    if (base) x = base[i];
    else x = mk<double>(i == (size_t)unit ? 1.0 : 0.0, 0.0);
    // sum_c U[i,c] coef[c] in the basis arithmetic, columns in chunks of eight (the
    // chunk's loads are issued before its products), then one subtraction in FP64
    cx<A> s = mk<A>(0, 0);
    for (int c0 = 0; c0 < k; c0 += 8) {
      cx<A> u[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (c0 + q < k) u[q] = as<A>(U[(size_t)(c0 + q) * ldu + i]);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (c0 + q < k) s = s + u[q] * sc[c0 + q];
    }
    x = x - as<double>(s);
    out[i] = x;
    if (i >= tail0) acc += x.x * x.x + x.y * x.y;
  }
  if (tailpart) {
    __shared__ double red[RED_TPB / 32];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < RED_TPB / 32; ++w) s += red[w];
      tailpart[blockIdx.x] = s;
    }
  }
}

// partial sums of |v[i]|^2 for i >= i0
__global__ void __launch_bounds__(RED_TPB) k_norm2(const c64* __restrict__ v, size_t N, size_t i0,
                                                   double* part) {
  __shared__ double red[RED_TPB / 32];
  double acc = 0.0;
  for (size_t i = i0 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    const c64 x = v[i];
    acc += x.x * x.x + x.y * x.y;
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < RED_TPB / 32; ++w) s += red[w];
    part[blockIdx.x] = s;
  }
}

// s = sum part[0..nb); optionally v *= 1/sqrt(s) on device (no host round trip)
__global__ void k_sum_parts(const double* __restrict__ part, int nb, double* out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += part[b];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    s = warp_sum(s);
    if (threadIdx.x == 0) *out = s;
  }
}

__global__ void k_scale_by_rnorm(c64* v, size_t N, const double* __restrict__ ss) {
  const double inv = 1.0 / sqrt(*ss);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x)
    v[i] = cscale(v[i], inv);
}

// new reflector column: u = (w with entries [0,j) zeroed, w[j] += add) * scale
template <typename UT>
__global__ void k_make_reflector(const c64* __restrict__ w, size_t N, int j, c64 add,
                                 double scale, UT* u) {
  using A = typename BasisArith<UT>::A;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    c64 x = (i < (size_t)j) ? mk<double>(0, 0) : w[i];
    if (i == (size_t)j) x = x + add;
    const c64 y = cscale(x, scale);
    u[i] = mk<A>((A)y.x, (A)y.y);
  }
}

// out = a - b
__global__ void k_sub(const c64* __restrict__ a, const c64* __restrict__ b, size_t N, c64* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = a[i] - b[i];
}

// out = x + y_pad - sum_c U[i,c] coef[c] where y_pad holds ny leading entries
template <typename UT>
__global__ void k_xupdate(const c64* __restrict__ x, const UT* __restrict__ U, size_t ldu,
                          const c64* __restrict__ coef, const c64* __restrict__ ypad, int k,
                          size_t N, c64* out) {
  using A = typename BasisArith<UT>::A;
  extern __shared__ unsigned char sx_raw[];
  c64* yp = reinterpret_cast<c64*>(sx_raw);                 // k entries
  cx<A>* sc2 = reinterpret_cast<cx<A>*>(sx_raw + sizeof(c64) * k);  // k entries
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    yp[c] = ypad[c];
    sc2[c] = as<A>(coef[c]);
  }
  __syncthreads();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    c64 v = x[i];
    if (i < (size_t)k) v = v + yp[i];
    cx<A> s = mk<A>(0, 0);
    for (int c0 = 0; c0 < k; c0 += 8) {
      cx<A> u[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (c0 + q < k) u[q] = as<A>(U[(size_t)(c0 + q) * ldu + i]);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (c0 + q < k) s = s + u[q] * sc2[c0 + q];
    }
    out[i] = v - as<double>(s);
  }
}

__global__ void k_add(const c64* __restrict__ a, const c64* __restrict__ b, size_t N, c64* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = a[i] + b[i];
}

// Small dense triangular products of the compact-WY representation (T upper
// triangular, column-major with leading dimension ld), one CTA.
// mode 0: out = T(0:k,0:k) * in;  mode 1: out = T(0:k,0:k)^H * in;
// mode 2: T(0:k, k) = -2 T(0:k,0:k) * in, T(k,k) = 2 (append a reflector)
__global__ void k_tri(c64* T, int ld, int k, const c64* __restrict__ in, c64* out, int mode) {
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    c64 s = mk<double>(0, 0);
    if (mode == 1) {
      for (int j = 0; j <= i; ++j) s = s + cconj(T[(size_t)i * ld + j]) * in[j];
    } else {
      for (int j = i; j < k; ++j) s = s + T[(size_t)j * ld + i] * in[j];
    }
    if (mode == 2) out[i] = cscale(s, -2.0);
    else out[i] = s;
  }
  if (mode == 2 && threadIdx.x == 0) out[k] = mk<double>(2.0, 0.0);
}

// The device loop's forms of k_tri, with the iteration index j read from the cycle state
// (same sums in the same order as k_tri):
// mode 0: out = T(0:k,0:k) * conj(Utop(j, 0:k)), k = j + 1 (the coefficients of
//         v = P1..Pj e_j = e_j - U T conj(Utop(j, :)));
// mode 1: out = T(0:k,0:k)^H * in, k = j + 1;
// mode 2: after the scalar step (j = the new column k): T(0:k, k) = -2 T(0:k,0:k) * in,
//         T(k,k) = 2, only when that step appended a reflector.
__global__ void k_tri_dyn(c64* T, int ld, const GmDev* __restrict__ gs,
                          const c64* __restrict__ in, c64* out, int mode) {
  const int j = gs->j;
  if (mode == 2 && !gs->refl_on) return;
  const int k = mode == 2 ? j : j + 1;
  if (mode == 2) out = T + (size_t)k * ld;
  const c64* __restrict__ ut = gs->Utop;
  const int ldu = gs->ld;
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    c64 s = mk<double>(0, 0);
    if (mode == 1) {
      for (int q = 0; q <= i; ++q) s = s + cconj(T[(size_t)i * ld + q]) * in[q];
    } else if (mode == 0) {
      for (int q = i; q < k; ++q) s = s + T[(size_t)q * ld + i] * cconj(ut[(size_t)q * ldu + j]);
    } else {
      for (int q = i; q < k; ++q) s = s + T[(size_t)q * ld + i] * in[q];
    }
    if (mode == 2) out[i] = cscale(s, -2.0);
    else out[i] = s;
  }
  if (mode == 2 && threadIdx.x == 0) out[k] = mk<double>(2.0, 0.0);
}

// k_make_reflector with the column, the head correction and the scale from the scalar
// step: column j of U (j the new iteration count) when that step appended a reflector
template <typename UT>
__global__ void k_make_reflector_dyn(const c64* __restrict__ w, size_t N,
                                     const GmDev* __restrict__ gs, UT* U) {
  using A = typename BasisArith<UT>::A;
  if (!gs->refl_on) return;
  const size_t j = (size_t)gs->j;
  const c64 add = gs->refl_add;
  const double scale = gs->refl_scale;
  UT* u = U + j * N;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    c64 x = (i < j) ? mk<double>(0, 0) : w[i];
    if (i == j) x = x + add;
    const c64 y = cscale(x, scale);
    u[i] = mk<A>((A)y.x, (A)y.y);
  }
}

__device__ __forceinline__ double cabs2(c64 z) { return z.x * z.x + z.y * z.y; }
__device__ __forceinline__ c64 csign(c64 d) {
  if (d.x == 0.0 && d.y == 0.0) return mk<double>(1.0, 0.0);
  const double a = hypot(d.x, d.y);
  return mk<double>(d.x / a, d.y / a);
}
__device__ __forceinline__ c64 cdivr(c64 z, double r) { return mk<double>(z.x / r, z.y / r); }

// The scalar work of one Householder GMRES iteration (gmres_custom.jl:129-171), in FP64 on
// the device, given the orthogonalised vector v = Pj..P1 A v_j (its head rows) and the
// squared norm alpha2 of its rows from initer on:
//   * the new reflector's head correction a = sign(v(initer)) * alpha and scale, and its
//     leading rows in Utop (the reflector itself is written by k_make_reflector_dyn);
//   * the earlier Givens rotations applied to the new column, a new rotation that zeroes
//     its subdiagonal, the rotated right-hand side w, the column of R;
//   * |w(initer+1)|, the residual estimate, into res[initer] and the state;
// and sets the WHILE node's condition: go on while the estimate is above tolb, the cycle
// has iterations left and the host asked for no early exit. Every path sets it, and the
// iteration count grows by one per call, so a loop ends after at most `inner` iterations.
// One warp: its lanes bring v's head and the earlier rotations into shared memory (when
// they fit), then lane 0 does the scalar work; the rotations form a chain.
constexpr int GM_SMEM_MAX = 768;  // head entries staged in shared memory (36 KB in all)
__global__ void k_gm_step(const c64* __restrict__ v_g, const double* __restrict__ alpha2p,
                          GmDev* gs, cudaGraphConditionalHandle cond, int use_cond) {
  __shared__ c64 s_v[GM_SMEM_MAX];
  __shared__ c64 s_J[2 * GM_SMEM_MAX];
  GmDev& g = *gs;
  const int j = g.j, initer = j + 1, inner = g.inner, ld = g.ld, headlen = g.headlen, n = g.n;
  const int nv = min(inner + 1, headlen);
  const bool staged = nv <= GM_SMEM_MAX && 2 * j <= 2 * GM_SMEM_MAX && j >= 0;
  if (staged) {
    for (int i = threadIdx.x; i < nv; i += blockDim.x) s_v[i] = v_g[i];
    for (int i = threadIdx.x; i < 2 * j; i += blockDim.x) s_J[i] = g.J[i];
    __syncthreads();
  }
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const c64* __restrict__ v = staged ? s_v : v_g;
  const c64* __restrict__ Jold = staged ? s_J : g.J;
  if (j < 0 || initer > inner) {
    g.refl_on = 0;
    if (use_cond) cudaGraphSetConditional(cond, 0u);
    return;
  }
  const c64 zero = mk<double>(0, 0);
  c64* __restrict__ ucol = g.Utop + (size_t)initer * ld;
  int refl = 0;
  c64 a = zero;
  if (initer != n) {
    const double alpha2 = *alpha2p;
    const double alpha = sqrt(alpha2);
    if (alpha != 0) {
      const c64 vj1 = v[initer];
      a = cscale(csign(vj1), alpha);
      const double nu2 = alpha2 - cabs2(vj1) + cabs2(vj1 + a);
      const double sc = 1.0 / sqrt(nu2);
      for (int i = 0; i < headlen; ++i)
        ucol[i] = i < initer ? zero : (i == initer ? cscale(v[i] + a, sc) : cscale(v[i], sc));
      g.refl_add = a;
      g.refl_scale = sc;
      refl = 1;
    }
  }
  if (!refl)
    for (int i = 0; i < headlen; ++i) ucol[i] = zero;
  g.refl_on = refl;
  // the new column before the rotations: v's head, with the reflector's rows below initer
  // zeroed and -a at initer
  auto vs = [&](int i) -> c64 {
    if (refl && i > initer) return zero;
    if (refl && i == initer) return mk<double>(-a.x, -a.y);
    return i < nv ? v[i] : zero;
  };
  c64* __restrict__ Rc = g.R + (size_t)j * inner;
  c64 cur = vs(0);
  for (int c = 0; c < j; ++c) {
    const c64 nxt = vs(c + 1);
    const c64 Jc = Jold[2 * c], Js = Jold[2 * c + 1];
    Rc[c] = cconj(Jc) * cur + cconj(Js) * nxt;
    const c64 t = Js * cur;
    cur = mk<double>(-t.x, -t.y) + Jc * nxt;
  }
  c64 vj = cur, vj1 = vs(j + 1);
  if (initer != n) {
    const double rho = sqrt(cabs2(vj) + cabs2(vj1));
    const c64 Jc = cdivr(vj, rho), Js = cdivr(vj1, rho);
    g.J[2 * j] = Jc;
    g.J[2 * j + 1] = Js;
    const c64 wj = g.wv[j];
    const c64 t = Js * wj;
    g.wv[j + 1] = mk<double>(-t.x, -t.y);
    g.wv[j] = cconj(Jc) * wj;
    vj = mk<double>(rho, 0.0);
    vj1 = zero;
  }
  Rc[j] = vj;
  if (j + 1 < inner) Rc[j + 1] = vj1;
  for (int i = j + 2; i < inner; ++i) Rc[i] = vs(i);
  const c64 w1 = g.wv[j + 1];
  const double normr = hypot(w1.x, w1.y);
  g.res[initer] = normr;
  g.normr = normr;
  g.j = initer;
  const bool go = normr > g.tolb && initer < inner && initer != n && !g.exit_now;
  if (use_cond) cudaGraphSetConditional(cond, go ? 1u : 0u);
}

__global__ void k_cast_down(const c64* __restrict__ a, size_t N, c32* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = ccast<float>(a[i]);
}

// ------------------------------- launchers ----------------------------------------

static inline unsigned g_stream(size_t n) {
  size_t g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  return (unsigned)g;
}

int red_blocks(size_t N) { return (int)g_stream(N); }

// multi-dot CTAs per column tile: at least 8 rows per thread, at most 2 CTAs per SM
static inline unsigned md_blocks(size_t N) {
  size_t g = (N + 8 * RED_TPB - 1) / (8 * RED_TPB);
  if (g > MD_BLOCKS_MAX) g = MD_BLOCKS_MAX;
  if (g < 1) g = 1;
  return (unsigned)g;
}

// returns the number of kernels launched
template <typename UT, typename VT>
static int multidot_t(const UT* U, size_t ldu, const VT* v, size_t N, int k, c64* partial,
                      c64* out, cudaStream_t st) {
  if (k <= 0) return 0;
  const unsigned nb = md_blocks(N);
  const int full = k / KB, rem = k - full * KB;
  if (full) k_multidot<KB, UT, VT><<<dim3(nb, full), RED_TPB, 0, st>>>(U, ldu, v, N, 0, partial);
  const int c0 = full * KB;
  switch (rem) {
    case 1: k_multidot<1, UT, VT><<<nb, RED_TPB, 0, st>>>(U, ldu, v, N, c0, partial); break;
    case 2: k_multidot<2, UT, VT><<<nb, RED_TPB, 0, st>>>(U, ldu, v, N, c0, partial); break;
    case 3: k_multidot<3, UT, VT><<<nb, RED_TPB, 0, st>>>(U, ldu, v, N, c0, partial); break;
    case 4: k_multidot<4, UT, VT><<<nb, RED_TPB, 0, st>>>(U, ldu, v, N, c0, partial); break;
    case 5: k_multidot<5, UT, VT><<<nb, RED_TPB, 0, st>>>(U, ldu, v, N, c0, partial); break;
    case 6: k_multidot<6, UT, VT><<<nb, RED_TPB, 0, st>>>(U, ldu, v, N, c0, partial); break;
    case 7: k_multidot<7, UT, VT><<<nb, RED_TPB, 0, st>>>(U, ldu, v, N, c0, partial); break;
    default: break;
  }
  k_reduce_cols<<<(k + 7) / 8, 256, 0, st>>>(partial, nb, k, out);
  return (full ? 1 : 0) + (rem ? 1 : 0) + 1;
}
int launch_multidot(const c64* U, size_t ldu, const c64* v, size_t N, int k, c64* partial,
                    c64* out, cudaStream_t st) {
  return multidot_t(U, ldu, v, N, k, partial, out, st);
}
int launch_multidot(const cff* U, size_t ldu, const c64* v, size_t N, int k, c64* partial,
                    c64* out, cudaStream_t st) {
  return multidot_t(U, ldu, v, N, k, partial, out, st);
}
int launch_multidot(const cff* U, size_t ldu, const cff* v, size_t N, int k, c64* partial,
                    c64* out, cudaStream_t st) {
  return multidot_t(U, ldu, v, N, k, partial, out, st);
}

template <typename UT>
static void multiaxpy_t(const UT* U, size_t ldu, const c64* base, int unit, const c64* coef,
                        int k, size_t N, c64* out, size_t tail0, double* tailpart,
                        cudaStream_t st) {
  using A = typename BasisArith<UT>::A;
  const unsigned nb = g_stream(N);
  k_multiaxpy<UT><<<nb, RED_TPB, sizeof(cx<A>) * (k > 0 ? k : 1), st>>>(
      U, ldu, base, unit, coef, k, N, out, tail0, tailpart);
}
void launch_multiaxpy(const c64* U, size_t ldu, const c64* base, int unit, const c64* coef,
                      int k, size_t N, c64* out, size_t tail0, double* tailpart,
                      cudaStream_t st) {
  multiaxpy_t(U, ldu, base, unit, coef, k, N, out, tail0, tailpart, st);
}
void launch_multiaxpy(const cff* U, size_t ldu, const c64* base, int unit, const c64* coef,
                      int k, size_t N, c64* out, size_t tail0, double* tailpart,
                      cudaStream_t st) {
  multiaxpy_t(U, ldu, base, unit, coef, k, N, out, tail0, tailpart, st);
}

void launch_norm2(const c64* v, size_t N, size_t i0, double* part, double* out, cudaStream_t st) {
  const unsigned nb = g_stream(N);
  k_norm2<<<nb, RED_TPB, 0, st>>>(v, N, i0, part);
  k_sum_parts<<<1, 1024, 0, st>>>(part, nb, out);
}

void launch_sum_parts(const double* part, int nb, double* out, cudaStream_t st) {
  k_sum_parts<<<1, 1024, 0, st>>>(part, nb, out);
}

void launch_scale_rnorm(c64* v, size_t N, const double* ss, cudaStream_t st) {
  k_scale_by_rnorm<<<g_stream(N), 256, 0, st>>>(v, N, ss);
}

void launch_make_reflector(const c64* w, size_t N, int j, c64 add, double scale, c64* u,
                           cudaStream_t st) {
  k_make_reflector<c64><<<g_stream(N), 256, 0, st>>>(w, N, j, add, scale, u);
}
void launch_make_reflector(const c64* w, size_t N, int j, c64 add, double scale, cff* u,
                           cudaStream_t st) {
  k_make_reflector<cff><<<g_stream(N), 256, 0, st>>>(w, N, j, add, scale, u);
}

void launch_sub(const c64* a, const c64* b, size_t N, c64* out, cudaStream_t st) {
  k_sub<<<g_stream(N), 256, 0, st>>>(a, b, N, out);
}

void launch_add(const c64* a, const c64* b, size_t N, c64* out, cudaStream_t st) {
  k_add<<<g_stream(N), 256, 0, st>>>(a, b, N, out);
}

// out += i * b (the imaginary-part convolutions of the Rcc operator joined to the real ones)
__global__ void k_add_i(const c64* __restrict__ b, size_t N, c64* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    const c64 u = out[i], v = b[i];
    out[i] = mk<double>(u.x - v.y, u.y + v.x);
  }
}

__global__ void k_set_scalar(double* p, double v) { *p = v; }

// *p = v in stream order (the value travels as a kernel argument, so no host buffer has to
// outlive the call)
void launch_set_scalar(double* p, double v, cudaStream_t st) { k_set_scalar<<<1, 1, 0, st>>>(p, v); }

void launch_add_i(const c64* b, size_t N, c64* out, cudaStream_t st) {
  k_add_i<<<g_stream(N), 256, 0, st>>>(b, N, out);
}

// flag |= 1 when a and b differ anywhere (bitwise on the doubles)
__global__ void k_differs(const c64* __restrict__ a, const c64* __restrict__ b, size_t N,
                          int* flag) {
  int d = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    const c64 u = a[i], v = b[i];
    d |= (__double_as_longlong(u.x) != __double_as_longlong(v.x)) |
         (__double_as_longlong(u.y) != __double_as_longlong(v.y));
  }
  if (__any_sync(0xffffffffu, d) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

void launch_differs(const c64* a, const c64* b, size_t N, int* flag, cudaStream_t st) {
  k_differs<<<g_stream(N), 256, 0, st>>>(a, b, N, flag);
}

void launch_tri(c64* T, int ld, int k, const c64* in, c64* out, int mode, cudaStream_t st) {
  k_tri<<<1, 256, 0, st>>>(T, ld, k, in, out, mode);
}

// The device loop's Arnoldi body around one operator application w = A v (the host
// loop's kernels in the same order, with the iteration index read on the device):
//   pre:  v = P1..Pj e_j = e_j - U T conj(Utop(j,:)), normalised (as the host loop does);
//   post: v = w - U T^H U^H w with the tail norm from row initer; the scalar step; the new
//         reflector and its column of T.
template <typename UT>
static int gm_pre_t(const GmBody& B, const UT* U) {
  using A = typename BasisArith<UT>::A;
  cudaStream_t st = B.st;
  const int* dj = &B.gs->j;
  k_tri_dyn<<<1, 256, 0, st>>>(B.T, B.ldT, B.gs, nullptr, B.coef, 0);
  k_multiaxpy<UT><<<g_stream(B.N), RED_TPB, sizeof(cx<A>) * (B.kmax + 1), st>>>(
      U, B.N, nullptr, 0, B.coef, 1, B.N, B.v, 0, nullptr, dj);
  launch_norm2(B.v, B.N, 0, B.red, B.scal, st);
  launch_scale_rnorm(B.v, B.N, B.scal, st);
  return 5;
}

template <typename UT>
static int gm_post_t(const GmBody& B, UT* U) {
  using A = typename BasisArith<UT>::A;
  cudaStream_t st = B.st;
  const int* dj = &B.gs->j;
  const unsigned nb = md_blocks(B.N);
  const unsigned tiles = (unsigned)((B.kmax + KB - 1) / KB);
  const unsigned rblk = (unsigned)((B.kmax + 7) / 8);
  // z = U(:,0:k)^H w, c = T^H z, v = w - U c with the tail norm from row initer
  k_multidot<KB, UT, c64, true><<<dim3(nb, tiles), RED_TPB, 0, st>>>(U, B.N, B.w, B.N, 0, B.part,
                                                                     dj, 1, 0);
  k_reduce_cols<<<rblk, 256, 0, st>>>(B.part, nb, 1, B.coef2, dj);
  k_tri_dyn<<<1, 256, 0, st>>>(B.T, B.ldT, B.gs, B.coef2, B.coef, 1);
  k_multiaxpy<UT><<<g_stream(B.N), RED_TPB, sizeof(cx<A>) * (B.kmax + 1), st>>>(
      U, B.N, B.w, 0, B.coef, 1, B.N, B.v, 1, B.red, dj);
  k_sum_parts<<<1, 1024, 0, st>>>(B.red, (int)g_stream(B.N), B.scal);
  k_gm_step<<<1, 32, 0, st>>>(B.v, B.scal, B.gs, B.cond, B.use_cond);
  // the new reflector u_k (k = the new iteration count) and T(0:k, k) = -2 T (U^H u_k)
  k_make_reflector_dyn<UT><<<g_stream(B.N), 256, 0, st>>>(B.v, B.N, B.gs, U);
  k_multidot<KB, UT, UT, true><<<dim3(nb, tiles), RED_TPB, 0, st>>>(U, B.N, U, B.N, 0, B.part, dj,
                                                                    0, B.N);
  k_reduce_cols<<<rblk, 256, 0, st>>>(B.part, nb, 0, B.coef2, dj);
  k_tri_dyn<<<1, 256, 0, st>>>(B.T, B.ldT, B.gs, B.coef2, nullptr, 2);
  return 10;
}

int gm_pre(const GmBody& B) { return B.U32 ? gm_pre_t<cff>(B, B.U32) : gm_pre_t<c64>(B, B.U); }
int gm_post(const GmBody& B) { return B.U32 ? gm_post_t<cff>(B, B.U32) : gm_post_t<c64>(B, B.U); }

void launch_xupdate(const c64* x, const c64* U, size_t ldu, const c64* coef, const c64* ypad,
                    int k, size_t N, c64* out, cudaStream_t st) {
  k_xupdate<c64><<<g_stream(N), 256, 2 * sizeof(c64) * (k > 0 ? k : 1), st>>>(x, U, ldu, coef,
                                                                             ypad, k, N, out);
}
void launch_xupdate(const c64* x, const cff* U, size_t ldu, const c64* coef, const c64* ypad,
                    int k, size_t N, c64* out, cudaStream_t st) {
  k_xupdate<cff><<<g_stream(N), 256, (sizeof(c64) + sizeof(cff)) * (k > 0 ? k : 1), st>>>(
      x, U, ldu, coef, ypad, k, N, out);
}

// ------------------------------------------------------------------------------------
// Allocation-free batched inner products (peec_multidot_noalloc)
//
// Some callers cannot call cudaMalloc at the point where they need these
// reductions: a host runtime whose device memory is entirely owned by its own
// pool allocator, or a latency-critical loop in which the implicit device
// synchronisation of cudaMalloc/cudaFree is not acceptable. For them the partial
// sums live in a fixed file-scope device array instead of caller- or
// context-owned scratch. It holds NOALLOC_BLOCKS x PEEC_NOALLOC_MAX_K complex
// doubles (1.25 MB) and stays resident on every GPU that loads this library until
// the process exits.
// ------------------------------------------------------------------------------------

constexpr int NOALLOC_BLOCKS = MD_BLOCKS_MAX;  // the multi-dot launcher's grid cap
static_assert(NOALLOC_BLOCKS >= MD_BLOCKS_MAX, "scratch smaller than the multi-dot grid");
static __device__ __align__(256) c64 g_noalloc_partials[(size_t)NOALLOC_BLOCKS * PEEC_NOALLOC_MAX_K];

// The array's device address belongs to the CUDA context that loaded this module. A
// cudaDeviceReset or a re-created primary context reloads the module and may move the
// array, so the looked-up address is cached per device together with the unique id of
// the context it was looked up in, and looked up again when the current context differs.
// The two driver calls are reached through the runtime, so the library needs no link
// against libcuda.
struct NoallocSlot {
  unsigned long long ctx_id = 0;
  void* addr = nullptr;
};
static std::mutex g_noalloc_mu;
static NoallocSlot g_noalloc_slot[256];
// held from launch to completion: calls on one device (any thread, any stream) take
// the shared array in turn
static std::mutex g_noalloc_run_mu[256];

typedef int (*drv_ctx_get_current_t)(void** ctx);
typedef int (*drv_ctx_get_id_t)(void* ctx, unsigned long long* id);
static std::once_flag g_drv_once;
static drv_ctx_get_current_t g_ctx_get_current = nullptr;
static drv_ctx_get_id_t g_ctx_get_id = nullptr;

static void resolve_driver_calls() {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
          cudaSuccess && q == cudaDriverEntryPointSuccess)
    g_ctx_get_current = (drv_ctx_get_current_t)f;
  f = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
          cudaSuccess && q == cudaDriverEntryPointSuccess)
    g_ctx_get_id = (drv_ctx_get_id_t)f;
  cudaGetLastError();
}

// the unique id of the calling thread's current context; 0 when it cannot be told
static unsigned long long current_context_id() {
  std::call_once(g_drv_once, resolve_driver_calls);
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  void* c = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&c) != 0 || !c) return 0;
  if (g_ctx_get_id(c, &id) != 0) return 0;
  return id;
}

}  // namespace peec

extern "C" int peec_multidot_noalloc(const void* U, int64_t ldu, const void* v, int64_t N, int k,
                                     void* out, void* stream) {
  using namespace peec;
  if (!U || !v || !out || N < 1 || ldu < N) {
    set_error("peec_multidot_noalloc: null pointer or N < 1 or ldu < N");
    return PEEC_ERR_BADARG;
  }
  if (k < 1 || k > PEEC_NOALLOC_MAX_K) {
    set_error("peec_multidot_noalloc: k = " + std::to_string(k) + " outside 1.." +
              std::to_string(PEEC_NOALLOC_MAX_K) + " (the fixed scratch holds " +
              std::to_string(PEEC_NOALLOC_MAX_K) + " columns)");
    return PEEC_ERR_BADARG;
  }
  int dev = 0;
  PEEC_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) {
    set_error("peec_multidot_noalloc: device ordinal out of range");
    return PEEC_ERR_BADARG;
  }
  void* scratch = nullptr;
  {
    // set-up once per device and context, with that device current: the host-side
    // name of the array is not a device address, so ask the runtime for it. The first
    // lookup in a context loads this module there, which places the array.
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocSlot& slot = g_noalloc_slot[dev];
    unsigned long long id = current_context_id();
    if (!slot.addr || id == 0 || slot.ctx_id != id) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(std::string("peec_multidot_noalloc: could not place the fixed scratch on "
                              "device ") + std::to_string(dev) + " (" + cudaGetErrorString(e) +
                  "); the first call on a device loads the library's device code there");
        return e == cudaErrorMemoryAllocation ? PEEC_ERR_OOM : PEEC_ERR_CUDA;
      }
      if (id == 0) id = current_context_id();  // the lookup made the primary context current
      slot.addr = p;
      slot.ctx_id = id;
    }
    scratch = slot.addr;
  }
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> run(g_noalloc_run_mu[dev]);
  // every partial[c][b] the reduction reads (c < k, b < grid) is written by this call's
  // multi-dot first, so the array needs no clearing between calls
  launch_multidot((const c64*)U, (size_t)ldu, (const c64*)v, (size_t)N, k, (c64*)scratch,
                  (c64*)out, st);
  PEEC_CUDA_TRY(cudaGetLastError());
  PEEC_CUDA_TRY(cudaStreamSynchronize(st));
  return PEEC_OK;
}
