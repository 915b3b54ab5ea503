// Shared-memory radix-2^q FFTs for power-of-two lengths.
//
// Forward transforms are decimation-in-frequency (natural order in, bit-reversed
// positions out); inverse transforms are decimation-in-time (bit-reversed in,
// natural out, unnormalised). A convolution therefore never permutes: spectra are
// produced by the same forward transform and multiply position-wise.
//
// Each thread takes 2^q elements of one sequence through q radix-2 stages in
// registers, so a length-256 transform costs three shared-memory round trips.
// Twiddles come from a table W[e] = exp(-2*pi*i*e/L), e < L/2.
#pragma once
#include "common.cuh"

namespace peec {

template <typename R, int Q, bool INV>
__device__ __forceinline__ void fft_group(cx<R>* seq, int estride, int s, int logL,
                                          const cx<R>* __restrict__ W, int c) {
  constexpr int RR = 1 << Q;
  const int lh = logL - s - Q;  // log2 of the element spacing inside the group
  const int hl = 1 << lh;
  const int bid = c >> lh;
  const int k = c & (hl - 1);
  const int start = (bid << (logL - s)) + k;
  cx<R> v[RR];
#pragma unroll
  for (int m = 0; m < RR; ++m) v[m] = seq[(start + m * hl) * estride];
  if (!INV) {
#pragma unroll
    for (int t = 0; t < Q; ++t) {
      const int half = RR >> (t + 1);
#pragma unroll
      for (int m = 0; m < RR; ++m) {
        if (!(m & half)) {
          cx<R> a = v[m], b = v[m + half];
          v[m] = a + b;
          const int e = (k + (m & (half - 1)) * hl) << (s + t);
          v[m + half] = (a - b) * W[e];
        }
      }
    }
  } else {
#pragma unroll
    for (int t = Q - 1; t >= 0; --t) {
      const int half = RR >> (t + 1);
#pragma unroll
      for (int m = 0; m < RR; ++m) {
        if (!(m & half)) {
          const int e = (k + (m & (half - 1)) * hl) << (s + t);
          cx<R> a = v[m], b = cmulc(v[m + half], W[e]);
          v[m] = a + b;
          v[m + half] = a - b;
        }
      }
    }
  }
#pragma unroll
  for (int m = 0; m < RR; ++m) seq[(start + m * hl) * estride] = v[m];
}

// Transforms nseq sequences (sequence i starts at buf + i*sstride, element stride
// estride) with the whole thread block. SEQ_MINOR maps consecutive threads to
// consecutive sequences (use when sequences are the contiguous direction).
// Ends with a __syncthreads().
template <typename R, bool INV, bool SEQ_MINOR>
__device__ void block_fft(cx<R>* buf, int nseq, int sstride, int estride, int logL,
                          const cx<R>* __restrict__ W) {
  if (logL == 0) {
    __syncthreads();
    return;
  }
  // stage groups: forward runs 3,3,..,rem from stage 0; inverse mirrors it
  int groups[16], ng = 0;
  for (int s = 0; s < logL;) {
    int q = (logL - s) >= 3 ? 3 : (logL - s);
    groups[ng++] = (s << 4) | q;
    s += q;
  }
  for (int gi = 0; gi < ng; ++gi) {
    const int g = INV ? groups[ng - 1 - gi] : groups[gi];
    const int s = g >> 4, q = g & 15;
    const int lper = logL - q;
    const int per = 1 << lper;
    const int total = nseq * per;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int sq, c;
      if (SEQ_MINOR) {
        sq = t % nseq;
        c = t / nseq;
      } else {
        sq = t >> lper;
        c = t & (per - 1);
      }
      cx<R>* seq = buf + sq * sstride;
      if (q == 3) fft_group<R, 3, INV>(seq, estride, s, logL, W, c);
      else if (q == 2) fft_group<R, 2, INV>(seq, estride, s, logL, W, c);
      else fft_group<R, 1, INV>(seq, estride, s, logL, W, c);
    }
    __syncthreads();
  }
}

}  // namespace peec
