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
//   k_ypass  forward / inverse FFT along y (32 or 16 consecutive kx per CTA)
//   k_zconv3 forward FFT along z of the three face families, 3x3 spectral product,
//            inverse FFT along z (one ky, a kx tile per CTA)
//   k_zconv1 same for one edge family with its real spectrum
//   k_xinv   inverse FFT along x and plain store into the compact output through the
//            lattice map (each compact index belongs to exactly one family)
// Only the occupied lattice octant is transformed in each pass (pruning). All tiles
// keep sequences contiguous in shared memory (element (pos, seq) at pos*rs + seq), so
// loads, stores and butterflies are bank-conflict free and index math is shifts.
// Spectra carry the 1/(Lx*Ly*Lz) normalisation and are stored (ky, kz, kx), kx fastest,
// in the transforms' bit-reversed position order.
#include <mutex>
#include <set>
#include <utility>

#include "ctx.hpp"
#include "fft.cuh"

namespace peec {

constexpr int TPB = 256;

// copy W_L[e] = exp(-2 pi i e / L) for e < n from the master table of length twmax
template <typename R>
__device__ void load_tw(cx<R>* dst, const cx<R>* __restrict__ master, int twmax, int L, int n) {
  const int step = twmax / L;
  for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = master[e * step];
}

// FFT of the 1<<LNS contiguous sequences of a tile: element (pos, seq) at buf[pos*rs + seq]
template <typename R, bool INV, int LNS>
__device__ void fft_cols(cx<R>* buf, int rs, int logL, const cx<R>* __restrict__ W) {
  if (logL == 0) {
    __syncthreads();
    return;
  }
  int groups[16], ng = 0;
  for (int s = 0; s < logL;) {
    const int q = (logL - s) >= 3 ? 3 : (logL - s);
    groups[ng++] = (s << 4) | q;
    s += q;
  }
  for (int gi = 0; gi < ng; ++gi) {
    const int g = INV ? groups[ng - 1 - gi] : groups[gi];
    const int s = g >> 4, q = g & 15;
    const int total = 1 << (logL - q + LNS);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int sq = t & ((1 << LNS) - 1);
      const int c = t >> LNS;
      cx<R>* seq = buf + sq;
      if (q == 3) fft_group<R, 3, INV>(seq, rs, s, logL, W, c);
      else if (q == 2) fft_group<R, 2, INV>(seq, rs, s, logL, W, c);
      else fft_group<R, 1, INV>(seq, rs, s, logL, W, c);
    }
    __syncthreads();
  }
}

// --------------------------------------------------------------------------- x passes

template <typename R, int LTY>
__global__ void __launch_bounds__(TPB) k_xfwd(const c64* __restrict__ xin,
                                              const int32_t* __restrict__ map, cx<R>* T, int Lx,
                                              int logLx, int Ly, int nx, int ny, int nz,
                                              const cx<R>* __restrict__ twm, int twmax) {
  constexpr int TY = 1 << LTY;
  extern __shared__ unsigned char smem_raw[];
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + (Lx > 1 ? Lx / 2 : 1);
  const int rs = TY + 1;
  const int y0 = blockIdx.x * TY, z = blockIdx.y;
  load_tw<R>(W, twm, twmax, Lx, Lx / 2);
  for (int p = threadIdx.x; p < TY << logLx; p += blockDim.x) {
    const int yy = p >> logLx, x = p & (Lx - 1);
    const int y = y0 + yy;
    cx<R> v = mk<R>(0, 0);
    if (y < ny && x < nx) {
      const int idx = map[((size_t)z * ny + y) * nx + x];
      if (idx >= 0) v = ccast<R>(xin[idx]);
    }
    buf[x * rs + yy] = v;
  }
  __syncthreads();
  fft_cols<R, false, LTY>(buf, rs, logLx, W);
  for (int p = threadIdx.x; p < TY << logLx; p += blockDim.x) {
    const int yy = p >> logLx, kx = p & (Lx - 1);
    const int y = y0 + yy;
    if (y < ny) T[((size_t)z * Ly + y) * Lx + kx] = buf[kx * rs + yy];
  }
}

template <typename R, int LTY>
__global__ void __launch_bounds__(TPB) k_xinv(const cx<R>* __restrict__ T, c64* yout,
                                              const int32_t* __restrict__ map, int Lx, int logLx,
                                              int Ly, int nx, int ny, int nz,
                                              const cx<R>* __restrict__ twm, int twmax) {
  constexpr int TY = 1 << LTY;
  extern __shared__ unsigned char smem_raw[];
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + (Lx > 1 ? Lx / 2 : 1);
  const int rs = TY + 1;
  const int y0 = blockIdx.x * TY, z = blockIdx.y;
  load_tw<R>(W, twm, twmax, Lx, Lx / 2);
  for (int p = threadIdx.x; p < TY << logLx; p += blockDim.x) {
    const int yy = p >> logLx, kx = p & (Lx - 1);
    const int y = y0 + yy;
    buf[kx * rs + yy] = (y < ny) ? T[((size_t)z * Ly + y) * Lx + kx] : mk<R>(0, 0);
  }
  __syncthreads();
  fft_cols<R, true, LTY>(buf, rs, logLx, W);
  for (int p = threadIdx.x; p < TY << logLx; p += blockDim.x) {
    const int yy = p >> logLx, x = p & (Lx - 1);
    const int y = y0 + yy;
    if (y >= ny || x >= nx) continue;
    const int idx = map[((size_t)z * ny + y) * nx + x];
    if (idx >= 0) {
      const cx<R> v = buf[x * rs + yy];
      yout[idx] = mk<double>((double)v.x, (double)v.y);
    }
  }
}

// --------------------------------------------------------------------------- y pass

// planes z < nz; rows y < n_in are read (zero padded to Ly), rows y < n_out written
template <typename R, bool INV, int LTX>
__global__ void __launch_bounds__(TPB) k_ypass(cx<R>* T, int Lx, int Ly, int logLy, int n_in,
                                               int n_out, const cx<R>* __restrict__ twm,
                                               int twmax) {
  constexpr int TX = 1 << LTX;
  extern __shared__ unsigned char smem_raw[];
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + (Ly > 1 ? Ly / 2 : 1);
  const int kx0 = blockIdx.x * TX, z = blockIdx.y;
  load_tw<R>(W, twm, twmax, Ly, Ly / 2);
  cx<R>* col = T + (size_t)z * Ly * Lx + kx0;
  for (int p = threadIdx.x; p < Ly << LTX; p += blockDim.x) {
    const int y = p >> LTX, tx = p & (TX - 1);
    buf[p] = (y < n_in) ? col[(size_t)y * Lx + tx] : mk<R>(0, 0);
  }
  __syncthreads();
  fft_cols<R, INV, LTX>(buf, TX, logLy, W);
  for (int p = threadIdx.x; p < n_out << LTX; p += blockDim.x) {
    const int y = p >> LTX, tx = p & (TX - 1);
    col[(size_t)y * Lx + tx] = buf[p];
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

template <typename R, int LTX>
__global__ void __launch_bounds__(TPB) k_zconv3(cx<R>* T0, cx<R>* T1, cx<R>* T2, int nz0, int nz1,
                                                int nz2, PSpec S, int Lx, int Ly, int Lz, int logLz,
                                                const cx<R>* __restrict__ twm, int twmax) {
  constexpr int TX = 1 << LTX;
  extern __shared__ unsigned char smem_raw[];
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* b0 = W + (Lz > 1 ? Lz / 2 : 1);
  cx<R>* b1 = b0 + (Lz << LTX);
  cx<R>* b2 = b1 + (Lz << LTX);
  const int kx0 = blockIdx.x * TX, ky = blockIdx.y;
  load_tw<R>(W, twm, twmax, Lz, Lz / 2);
  const size_t pl = (size_t)Ly * Lx;
  const size_t off = (size_t)ky * Lx + kx0;
  for (int p = threadIdx.x; p < Lz << LTX; p += blockDim.x) {
    const int z = p >> LTX, tx = p & (TX - 1);
    const size_t g = z * pl + off + tx;
    b0[p] = z < nz0 ? T0[g] : mk<R>(0, 0);
    b1[p] = z < nz1 ? T1[g] : mk<R>(0, 0);
    b2[p] = z < nz2 ? T2[g] : mk<R>(0, 0);
  }
  __syncthreads();
  fft_cols<R, false, LTX>(b0, TX, logLz, W);
  fft_cols<R, false, LTX>(b1, TX, logLz, W);
  fft_cols<R, false, LTX>(b2, TX, logLz, W);
  const R* s00 = reinterpret_cast<const R*>(S.s00);
  const R* s11 = reinterpret_cast<const R*>(S.s11);
  const R* s22 = reinterpret_cast<const R*>(S.s22);
  const cx<R>* s01 = reinterpret_cast<const cx<R>*>(S.s01);
  const cx<R>* s02 = reinterpret_cast<const cx<R>*>(S.s02);
  const cx<R>* s12 = reinterpret_cast<const cx<R>*>(S.s12);
  for (int p = threadIdx.x; p < Lz << LTX; p += blockDim.x) {
    const int kz = p >> LTX, tx = p & (TX - 1);
    const size_t si = ((size_t)ky * Lz + kz) * Lx + kx0 + tx;
    const cx<R> a0 = b0[p], a1 = b1[p], a2 = b2[p];
    const cx<R> c01 = s01[si], c02 = s02[si], c12 = s12[si];
    // Y_f = sum_g S_fg X_g with S_gf = conj(S_fg)
    b0[p] = cscale(a0, s00[si]) + c01 * a1 + c02 * a2;
    b1[p] = cmulc(a0, c01) + cscale(a1, s11[si]) + c12 * a2;
    b2[p] = cmulc(a0, c02) + cmulc(a1, c12) + cscale(a2, s22[si]);
  }
  __syncthreads();
  fft_cols<R, true, LTX>(b0, TX, logLz, W);
  fft_cols<R, true, LTX>(b1, TX, logLz, W);
  fft_cols<R, true, LTX>(b2, TX, logLz, W);
  for (int p = threadIdx.x; p < Lz << LTX; p += blockDim.x) {
    const int z = p >> LTX, tx = p & (TX - 1);
    const size_t g = z * pl + off + tx;
    if (z < nz0) T0[g] = b0[p];
    if (z < nz1) T1[g] = b1[p];
    if (z < nz2) T2[g] = b2[p];
  }
}

template <typename R, int LTX>
__global__ void __launch_bounds__(TPB) k_zconv1(cx<R>* T0, int nz0, const R* __restrict__ s00,
                                                int Lx, int Ly, int Lz, int logLz,
                                                const cx<R>* __restrict__ twm, int twmax) {
  constexpr int TX = 1 << LTX;
  extern __shared__ unsigned char smem_raw[];
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* b0 = W + (Lz > 1 ? Lz / 2 : 1);
  const int kx0 = blockIdx.x * TX, ky = blockIdx.y;
  load_tw<R>(W, twm, twmax, Lz, Lz / 2);
  const size_t pl = (size_t)Ly * Lx;
  const size_t off = (size_t)ky * Lx + kx0;
  for (int p = threadIdx.x; p < Lz << LTX; p += blockDim.x) {
    const int z = p >> LTX, tx = p & (TX - 1);
    b0[p] = z < nz0 ? T0[z * pl + off + tx] : mk<R>(0, 0);
  }
  __syncthreads();
  fft_cols<R, false, LTX>(b0, TX, logLz, W);
  for (int p = threadIdx.x; p < Lz << LTX; p += blockDim.x) {
    const int kz = p >> LTX, tx = p & (TX - 1);
    b0[p] = cscale(b0[p], s00[((size_t)ky * Lz + kz) * Lx + kx0 + tx]);
  }
  __syncthreads();
  fft_cols<R, true, LTX>(b0, TX, logLz, W);
  for (int p = threadIdx.x; p < nz0 << LTX; p += blockDim.x) {
    const int z = p >> LTX, tx = p & (TX - 1);
    T0[z * pl + off + tx] = b0[p];
  }
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

static inline int ltile(int logL, int want) { return logL < want ? logL : want; }

// one pass-class of launches; dispatches the compile-time tile widths
template <typename R>
struct Launch {
  static constexpr int LT = sizeof(R) == 8 ? 4 : 5;  // 16 (fp64) / 32 (fp32) kx per CTA
  static constexpr int LTY = 4;                      // 16 pencils per x-pass CTA

  static int xfwd(const Family& f, const c64* xin, const cx<R>* tw, int twmax, cudaStream_t st) {
    cx<R>* T = reinterpret_cast<cx<R>*>(f.T[sizeof(R) == 8 ? 0 : 1]);
    const int Lx = f.L[0];
    const size_t sm = sizeof(cx<R>) * ((Lx > 1 ? Lx / 2 : 1) + (size_t)Lx * ((1 << LTY) + 1));
    CTX_CHECK(smem_optin(k_xfwd<R, LTY>, sm));
    dim3 g((f.dims[1] + (1 << LTY) - 1) >> LTY, f.dims[2]);
    k_xfwd<R, LTY><<<g, TPB, sm, st>>>(xin, f.map, T, Lx, f.logL[0], f.L[1], f.dims[0], f.dims[1],
                                       f.dims[2], tw, twmax);
    return 0;
  }
  static int xinv(const Family& f, c64* yout, const cx<R>* tw, int twmax, cudaStream_t st) {
    cx<R>* T = reinterpret_cast<cx<R>*>(f.T[sizeof(R) == 8 ? 0 : 1]);
    const int Lx = f.L[0];
    const size_t sm = sizeof(cx<R>) * ((Lx > 1 ? Lx / 2 : 1) + (size_t)Lx * ((1 << LTY) + 1));
    CTX_CHECK(smem_optin(k_xinv<R, LTY>, sm));
    dim3 g((f.dims[1] + (1 << LTY) - 1) >> LTY, f.dims[2]);
    k_xinv<R, LTY><<<g, TPB, sm, st>>>(T, yout, f.map, Lx, f.logL[0], f.L[1], f.dims[0], f.dims[1],
                                       f.dims[2], tw, twmax);
    return 0;
  }
  template <bool INV, int LTX>
  static int ypass_t(const Family& f, const cx<R>* tw, int twmax, cudaStream_t st) {
    cx<R>* T = reinterpret_cast<cx<R>*>(f.T[sizeof(R) == 8 ? 0 : 1]);
    const int Ly = f.L[1];
    const size_t sm = sizeof(cx<R>) * ((Ly > 1 ? Ly / 2 : 1) + ((size_t)Ly << LTX));
    CTX_CHECK(smem_optin(k_ypass<R, INV, LTX>, sm));
    dim3 g(f.L[0] >> LTX, f.dims[2]);
    k_ypass<R, INV, LTX><<<g, TPB, sm, st>>>(T, f.L[0], Ly, f.logL[1], INV ? Ly : f.dims[1],
                                             INV ? f.dims[1] : Ly, tw, twmax);
    return 0;
  }
  template <bool INV>
  static int ypass(const Family& f, const cx<R>* tw, int twmax, cudaStream_t st) {
    switch (ltile(f.logL[0], LT)) {
      case 0: return ypass_t<INV, 0>(f, tw, twmax, st);
      case 1: return ypass_t<INV, 1>(f, tw, twmax, st);
      case 2: return ypass_t<INV, 2>(f, tw, twmax, st);
      case 3: return ypass_t<INV, 3>(f, tw, twmax, st);
      case 4: return ypass_t<INV, 4>(f, tw, twmax, st);
      default: return ypass_t<INV, LT>(f, tw, twmax, st);
    }
  }
  template <int LTX>
  static int zconv3_t(const Family* F, const PSpec& S, const cx<R>* tw, int twmax,
                      cudaStream_t st) {
    const int p = sizeof(R) == 8 ? 0 : 1;
    const int Lz = F[0].L[2];
    const size_t sm = sizeof(cx<R>) * ((Lz > 1 ? Lz / 2 : 1) + 3 * ((size_t)Lz << LTX));
    CTX_CHECK(smem_optin(k_zconv3<R, LTX>, sm));
    dim3 g(F[0].L[0] >> LTX, F[0].L[1]);
    k_zconv3<R, LTX><<<g, TPB, sm, st>>>(
        reinterpret_cast<cx<R>*>(F[0].T[p]), reinterpret_cast<cx<R>*>(F[1].T[p]),
        reinterpret_cast<cx<R>*>(F[2].T[p]), F[0].dims[2], F[1].dims[2], F[2].dims[2], S, F[0].L[0],
        F[0].L[1], Lz, F[0].logL[2], tw, twmax);
    return 0;
  }
  static int zconv3(const Family* F, const PSpec& S, const cx<R>* tw, int twmax, cudaStream_t st) {
    switch (ltile(F[0].logL[0], LT)) {
      case 0: return zconv3_t<0>(F, S, tw, twmax, st);
      case 1: return zconv3_t<1>(F, S, tw, twmax, st);
      case 2: return zconv3_t<2>(F, S, tw, twmax, st);
      case 3: return zconv3_t<3>(F, S, tw, twmax, st);
      case 4: return zconv3_t<4>(F, S, tw, twmax, st);
      default: return zconv3_t<LT>(F, S, tw, twmax, st);
    }
  }
  template <int LTX>
  static int zconv1_t(const Family& f, const void* s, const cx<R>* tw, int twmax,
                      cudaStream_t st) {
    const int p = sizeof(R) == 8 ? 0 : 1;
    const int Lz = f.L[2];
    const size_t sm = sizeof(cx<R>) * ((Lz > 1 ? Lz / 2 : 1) + ((size_t)Lz << LTX));
    CTX_CHECK(smem_optin(k_zconv1<R, LTX>, sm));
    dim3 g(f.L[0] >> LTX, f.L[1]);
    k_zconv1<R, LTX><<<g, TPB, sm, st>>>(reinterpret_cast<cx<R>*>(f.T[p]), f.dims[2],
                                         reinterpret_cast<const R*>(s), f.L[0], f.L[1], Lz,
                                         f.logL[2], tw, twmax);
    return 0;
  }
  static int zconv1(const Family& f, const void* s, const cx<R>* tw, int twmax, cudaStream_t st) {
    switch (ltile(f.logL[0], LT)) {
      case 0: return zconv1_t<0>(f, s, tw, twmax, st);
      case 1: return zconv1_t<1>(f, s, tw, twmax, st);
      case 2: return zconv1_t<2>(f, s, tw, twmax, st);
      case 3: return zconv1_t<3>(f, s, tw, twmax, st);
      case 4: return zconv1_t<4>(f, s, tw, twmax, st);
      default: return zconv1_t<LT>(f, s, tw, twmax, st);
    }
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
