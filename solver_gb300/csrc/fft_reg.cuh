// Register-resident radix-2^q FFT groups for the circulant passes.
//
// A length-L = 2^n transform is split into groups of q <= 4 radix-2 stages. A forward
// (decimation-in-frequency) group over the elements x_m = seq[start + m*hl],
// m < 2^q, of a sub-transform of size M = L >> s is
//   y_j = W_M^(k*j) * sum_m x_m w_(2^q)^(m*j),  stored at start + brev_q(j)*hl,
// i.e. a small DFT with constant twiddles (16th roots of unity) followed by one table
// twiddle per output. Chaining the groups in stage order gives the natural-in,
// bit-reversed-out DIF transform; the inverse runs the conjugate-transposed groups in
// reverse order (decimation in time, bit-reversed in, natural out, unnormalised).
// These are exactly the transforms the spectra are built with, so a convolution never
// permutes.
//
// Pass kernels keep the first group's inputs and the last group's outputs in
// registers, reading and writing global memory directly; only the middle groups go
// through shared memory.
#pragma once
#include <type_traits>

#include "common.cuh"

namespace peec {

// cos(a*pi/8), a in [0, 16)
__host__ __device__ constexpr double cospi8(int a) {
  return a == 0    ? 1.0
         : a == 1  ? 0.92387953251128675613
         : a == 2  ? 0.70710678118654752440
         : a == 3  ? 0.38268343236508977173
         : a == 4  ? 0.0
         : a == 5  ? -0.38268343236508977173
         : a == 6  ? -0.70710678118654752440
         : a == 7  ? -0.92387953251128675613
         : a == 8  ? -1.0
         : a == 9  ? -0.92387953251128675613
         : a == 10 ? -0.70710678118654752440
         : a == 11 ? -0.38268343236508977173
         : a == 12 ? 0.0
         : a == 13 ? 0.38268343236508977173
         : a == 14 ? 0.70710678118654752440
                   : 0.92387953251128675613;
}
__host__ __device__ constexpr double sinpi8(int a) { return cospi8((a + 12) & 15); }

__host__ __device__ constexpr int brevq(int r, int q) {
  int o = 0;
  for (int i = 0; i < q; ++i) o |= ((r >> i) & 1) << (q - 1 - i);
  return o;
}

// v * exp(-i*a*pi/8) (forward) or v * exp(+i*a*pi/8) (INV); a is a compile-time
// constant after unrolling, so the quarter turns reduce to swaps and negations
template <typename R, bool INV>
__device__ __forceinline__ cx<R> rot16(const cx<R>& v, int a) {
  a &= 15;
  if (a == 0) return v;
  if (a == 8) return mk<R>(-v.x, -v.y);
  if (a == 4) return INV ? mk<R>(-v.y, v.x) : mk<R>(v.y, -v.x);
  if (a == 12) return INV ? mk<R>(v.y, -v.x) : mk<R>(-v.y, v.x);
  const R c = (R)cospi8(a);
  const R s = INV ? (R)sinpi8(a) : (R)(-sinpi8(a));
  return mk<R>(v.x * c - v.y * s, v.x * s + v.y * c);
}

// forward DFT of 2^Q registers: natural order in, register r holds output brev_Q(r)
template <typename R, int Q>
__device__ __forceinline__ void dft_dif(cx<R>* v) {
  constexpr int N = 1 << Q;
#pragma unroll
  for (int t = 0; t < Q; ++t) {
    const int half = N >> (t + 1);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (!(m & half)) {
        const cx<R> a = v[m], b = v[m + half];
        v[m] = a + b;
        v[m + half] = rot16<R, false>(a - b, ((m & (half - 1)) << t) * (16 / N));
      }
    }
  }
}

// conjugate transpose of dft_dif: register r holds input brev_Q(r), natural order out
template <typename R, int Q>
__device__ __forceinline__ void dft_dit(cx<R>* v) {
  constexpr int N = 1 << Q;
#pragma unroll
  for (int t = Q - 1; t >= 0; --t) {
    const int half = N >> (t + 1);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (!(m & half)) {
        const cx<R> a = v[m];
        const cx<R> b = rot16<R, true>(v[m + half], ((m & (half - 1)) << t) * (16 / N));
        v[m] = a + b;
        v[m + half] = a - b;
      }
    }
  }
}

// group twiddles W_L^((k*brev_Q(r)) << s), W the full-length table of this transform;
// conjugated for the inverse (applied before dft_dit)
template <typename R, int Q, bool INV>
__device__ __forceinline__ void group_twiddle(cx<R>* v, int k, int s, const cx<R>* W) {
  if (k == 0) return;
#pragma unroll
  for (int r = 1; r < (1 << Q); ++r) {
    const cx<R> w = W[(k * brevq(r, Q)) << s];
    v[r] = INV ? cmulc(v[r], w) : v[r] * w;
  }
}

// a length-2^n transform as groups q[0..ng) in forward stage order
struct AxPlan {
  int n;
  int ng;
  int q[12];
};

// single: largest n done as one register group; first/last: caps of the first and last
// group when there are several; middle groups take at most 3 stages
inline AxPlan make_plan(int n, int single, int first, int last) {
  AxPlan p{};
  p.n = n;
  if (n <= single) {
    p.ng = 1;
    p.q[0] = n;
    return p;
  }
  int ql = last < n - 1 ? last : n - 1;
  int q0 = first < n - ql ? first : n - ql;
  int rest = n - ql - q0;
  p.q[p.ng++] = q0;
  while (rest > 0) {
    const int q = rest >= 3 ? 3 : rest;
    p.q[p.ng++] = q;
    rest -= q;
  }
  p.q[p.ng++] = ql;
  return p;
}

__device__ __forceinline__ int plan_s(const AxPlan& p, int g) {
  int s = 0;
  for (int i = 0; i < g; ++i) s += p.q[i];
  return s;
}

// one middle group over a shared-memory tile: element (pos, col) at buf[pos*rs + col],
// 2^LC columns, sequences of length 2^n, group at stage offset s
template <typename R, int Q, bool INV, int LC>
__device__ __forceinline__ void smem_group(cx<R>* buf, int rs, int n, int s, const cx<R>* W) {
  constexpr int N = 1 << Q;
  const int lh = n - s - Q;
  const int tasks = 1 << (n - Q + LC);
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int col = t & ((1 << LC) - 1);
    const int c = t >> LC;
    const int k = c & ((1 << lh) - 1);
    const int start = ((c >> lh) << (n - s)) + k;
    cx<R> v[N];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = buf[(start + (r << lh)) * rs + col];
    if (!INV) {
      dft_dif<R, Q>(v);
      group_twiddle<R, Q, false>(v, k, s, W);
    } else {
      group_twiddle<R, Q, true>(v, k, s, W);
      dft_dit<R, Q>(v);
    }
#pragma unroll
    for (int r = 0; r < N; ++r) buf[(start + (r << lh)) * rs + col] = v[r];
  }
}

// runtime group size -> compile-time instantiation, at most MAXQ (plans never exceed
// the cap a kernel is built for, so larger register groups are never compiled in)
template <int V>
using qconst = std::integral_constant<int, V>;

template <int MAXQ, typename F>
__device__ __forceinline__ void qswitch(int q, F&& f) {
  if (q <= 0) {
    f(qconst<0>{});
  } else if (q == 1) {
    if constexpr (MAXQ >= 1) f(qconst<1>{});
  } else if (q == 2) {
    if constexpr (MAXQ >= 2) f(qconst<2>{});
  } else if (q == 3) {
    if constexpr (MAXQ >= 3) f(qconst<3>{});
  } else {
    if constexpr (MAXQ >= 4) f(qconst<4>{});
  }
}

// middle groups take at most 3 stages
template <typename R, bool INV, int LC>
__device__ __forceinline__ void smem_group_q(cx<R>* buf, int rs, int q, int n, int s,
                                             const cx<R>* W) {
  qswitch<3>(q, [&](auto QC) { smem_group<R, decltype(QC)::value, INV, LC>(buf, rs, n, s, W); });
}

// the middle groups of a plan (forward in stage order, inverse reversed), each
// followed by a barrier
template <typename R, bool INV, int LC>
__device__ void middle_groups(cx<R>* buf, int rs, const AxPlan& p, const cx<R>* W) {
  if (!INV) {
    int s = p.q[0];
    for (int g = 1; g + 1 < p.ng; ++g) {
      smem_group_q<R, false, LC>(buf, rs, p.q[g], p.n, s, W);
      s += p.q[g];
      __syncthreads();
    }
  } else {
    int s = p.n - p.q[p.ng - 1];
    for (int g = p.ng - 2; g >= 1; --g) {
      s -= p.q[g];
      smem_group_q<R, true, LC>(buf, rs, p.q[g], p.n, s, W);
      __syncthreads();
    }
  }
}

// full-length twiddle table of a length-L transform from the master table
template <typename R>
__device__ __forceinline__ void load_twiddles(cx<R>* W, const cx<R>* __restrict__ master,
                                              int twmax, int L) {
  const int step = twmax / L;
  for (int e = threadIdx.x; e < L; e += blockDim.x) W[e] = master[e * step];
}

}  // namespace peec
