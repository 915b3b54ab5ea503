// Numeric refactorisation of SS = Yle + A' diag(1/DZ) A + jw Gamma diag(1/P) Gamma' on the
// device, per frequency, in the pattern and permutations of a host factorisation done
// once (the reference factorises with UMFPACK on the host at every frequency,
// FFT_solver_QS_S_type.jl:118-119). SS's structure does not depend on the frequency, so
// the fill of Pr SS Pc = L U in a fixed pivot order does not either; SS is close to
// diagonally dominant (off-diagonal row sums at most ~1.04 of the diagonal's magnitude
// on the benchmark grids), so keeping the first frequency's pivot order is stable. Every
// pivot is checked: zero or non-finite pivots set an error word the host reports.
//
//   assemble: every slot of L (off-diagonal), of the diagonal D and of U (off-diagonal)
//             is the sum of its SS contributions, in a fixed order per slot (edges'
//             +-1/DZ, surfaces' jw/P, Yle entries); slots of fill start at zero
//   rows:     up-looking, one thread per permuted row, rows of one L level per launch
//             (a row depends on the rows of its L pattern, all of earlier levels):
//               for k in L(p,:) in increasing order: L(p,k) = w(k) / D(k);
//                 w(j) -= L(p,k) U(k,j) for j in U(k,:)   (targets precomputed)
//             then D(p) is final; U.dinv(p) = 1 / D(p), L's diagonal stays 1
#include "ctx.hpp"

namespace peec {

// contribution codes of asm_src: type in the top two bits, index below
constexpr uint32_t RF_EDGE_DIAG = 0u, RF_EDGE_OFF = 1u, RF_SURF = 2u, RF_YLE = 3u;

__global__ void k_rf_assemble(int64_t nslot, const int64_t* __restrict__ ptr,
                              const uint32_t* __restrict__ src, const c64* __restrict__ DZ,
                              const double* __restrict__ invP, const c64* __restrict__ yle,
                              double w, int64_t nL, int64_t n, c64* Lval, c64* D, c64* Uval) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nslot;
       s += (int64_t)gridDim.x * blockDim.x) {
    c64 acc = mk<double>(0, 0);
    for (int64_t q = ptr[s]; q < ptr[s + 1]; ++q) {
      const uint32_t code = src[q];
      const uint32_t t = code >> 30, i = code & 0x3fffffffu;
      if (t == RF_EDGE_DIAG || t == RF_EDGE_OFF) {
        const c64 d = DZ[i];
        const double den = d.x * d.x + d.y * d.y;
        const c64 iz = mk<double>(d.x / den, -d.y / den);
        acc = t == RF_EDGE_DIAG ? acc + iz : acc - iz;
      } else if (t == RF_SURF) {
        acc = acc + mk<double>(0.0, w * invP[i]);
      } else {
        acc = acc + yle[i];
      }
    }
    if (s < nL) Lval[s] = acc;
    else if (s < nL + n) D[s - nL] = acc;
    else Uval[s - nL - n] = acc;
  }
}

// upd_tgt codes: -1 the row's own diagonal; bit 30 set: U.val index (low 30 bits); else
// L.val index
__global__ void k_rf_rows(const int32_t* __restrict__ rows, int nrows, SfTri L, SfTri U, c64* D,
                          const int32_t* __restrict__ upd_off, const int32_t* __restrict__ upd_tgt,
                          int* err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  const int p = rows[t];
  c64* Lval = const_cast<c64*>(L.val);
  c64* Uval = const_cast<c64*>(U.val);
  for (int q = L.ptr[p]; q < L.ptr[p + 1]; ++q) {
    const int k = L.col[q];
    const c64 dk = D[k];
    const double den = dk.x * dk.x + dk.y * dk.y;
    const c64 w = Lval[q];
    const c64 l = mk<double>((w.x * dk.x + w.y * dk.y) / den, (w.y * dk.x - w.x * dk.y) / den);
    Lval[q] = l;
    const int u0 = U.ptr[k];
    for (int e = upd_off[q]; e < upd_off[q + 1]; ++e) {
      const int tg = upd_tgt[e];
      const c64 v = l * Uval[u0 + (e - upd_off[q])];
      if (tg < 0) D[p] = D[p] - v;
      else if (tg & 0x40000000) Uval[tg & 0x3fffffff] = Uval[tg & 0x3fffffff] - v;
      else Lval[tg] = Lval[tg] - v;
    }
  }
  const c64 d = D[p];
  const double den = d.x * d.x + d.y * d.y;
  if (!(den > 0.0) || !isfinite(den)) atomicExch(err, 1);
  const_cast<c64*>(U.dinv)[p] = mk<double>(d.x / den, -d.y / den);
  const_cast<c64*>(L.dinv)[p] = mk<double>(1.0, 0.0);
}

int refactor_launch(const RefactorPlan& R, const SfTri& L, const SfTri& U, c64* Lval, c64* Uval,
                    const c64* DZ, const double* invP, const c64* yle, double w, int* err,
                    cudaStream_t st) {
  const int64_t nslot = R.nL + R.n + R.nU;
  int64_t blocks = (nslot + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_rf_assemble<<<(unsigned)blocks, 256, 0, st>>>(nslot, R.asm_ptr, R.asm_src, DZ, invP, yle, w,
                                                  R.nL, R.n, Lval, R.D, Uval);
  int launches = 1;
  for (size_t l = 0; l + 1 < R.lvl_off.size(); ++l) {
    const int a = R.lvl_off[l], b = R.lvl_off[l + 1];
    if (b <= a) continue;
    k_rf_rows<<<(b - a + 127) / 128, 128, 0, st>>>(R.rows + a, b - a, L, U, R.D, R.upd_off,
                                                   R.upd_tgt, err);
    ++launches;
  }
  PEEC_CUDA_TRY(cudaGetLastError());
  return launches;
}

// The per-frequency edge impedances DZ on the device (FFT_solver_QS_S_type.jl:105-114):
//   Z_self = sum over the four edge halves of 1/(1/R + jw Cd), R, or 1/(jw Cd) where only
//            one of them is present (compute_Z_self.jl:1-15);
//   Zs     = escal_R * Zs0 * sqrt(w / escal_freq) (real part);
//   on surface edges: Z_self keeps only its imaginary part where Zs > Re(Z_self), Zs is
//            dropped where Zs < Re(Z_self);
//   DZ     = Z_self + Zs + jw Lp_self.
// The arithmetic is that of the host state (frequency.FrequencyState): the same
// operations on doubles, one edge per thread.
__global__ void k_edge_dz(int64_t m, const double* __restrict__ R4, const double* __restrict__ Cd4,
                          const double* __restrict__ Lpd, const double* __restrict__ Zs0,
                          const uint8_t* __restrict__ surf, double escal_R, double sq, double w,
                          c64* DZ) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m;
       e += (int64_t)gridDim.x * blockDim.x) {
    double zr = 0.0, zi = 0.0;
    for (int a = 0; a < 4; ++a) {
      const double r = R4[4 * e + a], cd = Cd4[4 * e + a];
      if (r != 0.0 && cd != 0.0) {
        // 1 / (1/r + j w cd)
        const double p = 1.0 / r, q = w * cd;
        const double den = p * p + q * q;
        zr += p / den;
        zi += -q / den;
      } else if (r != 0.0) {
        zr += r;
      } else if (cd != 0.0) {
        // 1 / (j w cd) = -j / (w cd)
        zi += -1.0 / (w * cd);
      }
    }
    double zs = escal_R * (Zs0[e] * sq);
    if (surf[e]) {
      const double d = zs - zr;
      if (d > 0) zr = 0.0;
      else if (d < 0) zs = 0.0;
    }
    DZ[e] = mk<double>(zr + zs, zi + w * Lpd[e]);
  }
}

void launch_edge_dz(int64_t m, const double* R4, const double* Cd4, const double* Lpd,
                    const double* Zs0, const uint8_t* surf, double escal_R, double sq, double w,
                    c64* DZ, cudaStream_t st) {
  int64_t b = (m + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  k_edge_dz<<<(unsigned)b, 256, 0, st>>>(m, R4, Cd4, Lpd, Zs0, surf, escal_R, sq, w, DZ);
}

}  // namespace peec
