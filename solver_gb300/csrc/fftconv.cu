// Pruned circulant-convolution kernels for the voxel Lp / P Toeplitz blocks.
//
// One block application y_out += K * x_in on lattices of extents nb (input) and na
// (output) runs as three kernels over an Lx x Ly x Lz circulant grid:
//   k_xfwd : gather x_in through the lattice map, zero-pad, forward FFT along x
//            (TY pencils per CTA), store transposed T1[kx][z][y] so that each kx
//            plane is contiguous for the next pass;
//   k_yz   : per kx plane (and ky sub-block r of R): forward y-FFT, then per ky row
//            forward z-FFT, multiply by the spectrum, inverse z-FFT, and the
//            inverse y-FFT of the output columns; store T4[r][kx][z][y];
//   k_xinv : sum the R sub-block partials, inverse x-FFT, keep the na output
//            points and accumulate them into y_out through the output map.
// Zero padding is never materialised in global memory and only the lattice
// octant is transformed in each direction (pruning). The spectrum carries the
// 1/(Lx*Ly*Lz) normalisation.
#include "ctx.hpp"
#include "fft.cuh"

namespace peec {

constexpr int TPB = 256;

template <typename R>
struct TwT;
template <>
struct TwT<double> {
  using T = c64;
};
template <>
struct TwT<float> {
  using T = c32;
};

// copy W_L[e] = exp(-2 pi i e / L) for e < n from the master table of length twmax
template <typename R>
__device__ void load_tw(cx<R>* dst, const cx<R>* __restrict__ master, int twmax, int L, int n) {
  const int step = twmax / L;
  for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = master[e * step];
}

template <typename R, int TY>
__global__ void __launch_bounds__(TPB) k_xfwd(const c64* __restrict__ xin,
                                              const int32_t* __restrict__ in_map, cx<R>* T1,
                                              int Lx, int logLx, int nbx, int nby, int nbz,
                                              const cx<R>* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + (Lx / 2 > 0 ? Lx / 2 : 1);
  const int sst = Lx + 1;
  const int y0 = blockIdx.x * TY;
  const int z = blockIdx.y;
  load_tw<R>(W, twm, twmax, Lx, Lx / 2);
  for (int p = threadIdx.x; p < TY * Lx; p += blockDim.x) {
    const int yy = p / Lx, x = p - yy * Lx;
    const int y = y0 + yy;
    cx<R> v = mk<R>(0, 0);
    if (y < nby && x < nbx) {
      const int idx = in_map[((size_t)z * nby + y) * nbx + x];
      if (idx >= 0) v = ccast<R>(xin[idx]);
    }
    buf[yy * sst + x] = v;
  }
  __syncthreads();
  block_fft<R, false, false>(buf, TY, sst, 1, logLx, W);
  for (int p = threadIdx.x; p < TY * Lx; p += blockDim.x) {
    const int kx = p / TY, yy = p - kx * TY;
    const int y = y0 + yy;
    if (y < nby) T1[((size_t)kx * nbz + z) * nby + y] = buf[yy * sst + kx];
  }
}

template <typename R, typename SR, bool CPLX>
__global__ void __launch_bounds__(TPB) k_yz(const cx<R>* __restrict__ T1, cx<R>* T4,
                                            const SR* __restrict__ spec, int conj, int Lx,
                                            int Ly, int logLy, int Lz, int logLz, int logR,
                                            int nby, int nbz, int nay, int naz,
                                            const cx<R>* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  const int R_ = 1 << logR;
  const int Lyl = Ly >> logR, logLyl = logLy - logR;
  cx<R>* Wy = reinterpret_cast<cx<R>*>(smem_raw);                 // W_{Lyl}, Lyl/2
  cx<R>* Wz = Wy + (Lyl / 2 > 0 ? Lyl / 2 : 1);                    // W_{Lz}, Lz/2
  cx<R>* Wf = Wz + (Lz / 2 > 0 ? Lz / 2 : 1);                      // W_{Ly}, Ly (only if R>1)
  cx<R>* plane = Wf + (R_ > 1 ? Ly : 0);                          // Lyl rows x (Lz+1)
  const int rs = Lz + 1;
  const int kx = blockIdx.x;
  const int r = blockIdx.y;
  const int rho = brev(r, logR);
  load_tw<R>(Wy, twm, twmax, Lyl, Lyl / 2);
  load_tw<R>(Wz, twm, twmax, Lz, Lz / 2);
  if (R_ > 1) load_tw<R>(Wf, twm, twmax, Ly, Ly);
  __syncthreads();
  // load the kx plane, folding the first logR DIF stages for sub-block r:
  // y_r[n] = W_Ly^{n*rho} * sum_q x[n + q*Lyl] * W_Ly^{q*rho*Lyl}
  const cx<R>* src = T1 + (size_t)kx * nbz * nby;
  for (int p = threadIdx.x; p < Lyl * Lz; p += blockDim.x) {
    const int z = p / Lyl, n = p - z * Lyl;
    cx<R> v = mk<R>(0, 0);
    if (z < nbz) {
      if (R_ == 1) {
        if (n < nby) v = src[(size_t)z * nby + n];
      } else {
        for (int q = 0; q < R_; ++q) {
          const int y = n + q * Lyl;
          if (y < nby) v = v + src[(size_t)z * nby + y] * Wf[(q * rho * Lyl) & (Ly - 1)];
        }
        v = v * Wf[(n * rho) & (Ly - 1)];
      }
    }
    plane[n * rs + z] = v;
  }
  __syncthreads();
  block_fft<R, false, true>(plane, nbz, 1, rs, logLyl, Wy);          // y forward
  block_fft<R, false, false>(plane, Lyl, rs, 1, logLz, Wz);          // z forward
  const size_t sbase = ((size_t)kx * Ly + (size_t)r * Lyl) * Lz;
  for (int p = threadIdx.x; p < Lyl * Lz; p += blockDim.x) {
    const int n = p / Lz, z = p - n * Lz;
    const size_t si = sbase + (size_t)n * Lz + z;
    cx<R> v = plane[n * rs + z];
    if (CPLX) {
      const cx<SR> s = reinterpret_cast<const cx<SR>*>(spec)[si];
      cx<R> sv = mk<R>((R)s.x, conj ? -(R)s.y : (R)s.y);
      v = v * sv;
    } else {
      v = cscale(v, (R)spec[si]);
    }
    plane[n * rs + z] = v;
  }
  __syncthreads();
  block_fft<R, true, false>(plane, Lyl, rs, 1, logLz, Wz);           // z inverse
  block_fft<R, true, true>(plane, naz, 1, rs, logLyl, Wy);           // y inverse
  cx<R>* dst = T4 + ((size_t)r * Lx + kx) * naz * nay;
  for (int p = threadIdx.x; p < naz * nay; p += blockDim.x) {
    const int z = p / nay, j = p - z * nay;
    cx<R> v = plane[(j & (Lyl - 1)) * rs + z];
    if (R_ > 1) v = cmulc(v, Wf[(j * rho) & (Ly - 1)]);
    dst[(size_t)z * nay + j] = v;
  }
}

template <typename R, int TY>
__global__ void __launch_bounds__(TPB) k_xinv(const cx<R>* __restrict__ T4, c64* yout,
                                              const int32_t* __restrict__ out_map, int Lx,
                                              int logLx, int R_, int nax, int nay, int naz,
                                              const cx<R>* __restrict__ twm, int twmax) {
  extern __shared__ unsigned char smem_raw[];
  cx<R>* W = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf = W + (Lx / 2 > 0 ? Lx / 2 : 1);
  const int sst = Lx + 1;
  const int y0 = blockIdx.x * TY;
  const int z = blockIdx.y;
  load_tw<R>(W, twm, twmax, Lx, Lx / 2);
  const size_t pstride = (size_t)Lx * naz * nay;
  for (int p = threadIdx.x; p < TY * Lx; p += blockDim.x) {
    const int kx = p / TY, yy = p - kx * TY;
    const int y = y0 + yy;
    cx<R> v = mk<R>(0, 0);
    if (y < nay) {
      const size_t o = ((size_t)kx * naz + z) * nay + y;
      for (int r = 0; r < R_; ++r) v = v + T4[o + r * pstride];
    }
    buf[yy * sst + kx] = v;
  }
  __syncthreads();
  block_fft<R, true, false>(buf, TY, sst, 1, logLx, W);
  for (int p = threadIdx.x; p < TY * nax; p += blockDim.x) {
    const int yy = p / nax, x = p - yy * nax;
    const int y = y0 + yy;
    if (y >= nay) continue;
    const int idx = out_map[((size_t)z * nay + y) * nax + x];
    if (idx >= 0) {
      const cx<R> v = buf[yy * sst + x];
      c64 o = yout[idx];
      o.x += (double)v.x;
      o.y += (double)v.y;
      yout[idx] = o;
    }
  }
}

template <typename R>
static int conv_apply_t(const ConvApp& a, const Spectrum& S, const int32_t* in_map,
                        const int32_t* out_map, const c64* xin, c64* yout, const cx<R>* tw,
                        int twmax, cudaStream_t st, cudaEvent_t* evs) {
  constexpr int TY = 16;
  const int prec = sizeof(R) == 8 ? 0 : 1;
  const int Lx = a.L[0], Ly = a.L[1], Lz = a.L[2];
  cx<R>* T1 = reinterpret_cast<cx<R>*>(a.T1[prec]);
  cx<R>* T4 = reinterpret_cast<cx<R>*>(a.T4[prec]);
  size_t sm_x = sizeof(cx<R>) * ((Lx / 2 > 0 ? Lx / 2 : 1) + (size_t)TY * (Lx + 1));
  dim3 gx((a.nb[1] + TY - 1) / TY, a.nb[2]);
  if (evs) cudaEventRecord(evs[0], st);
  k_xfwd<R, TY><<<gx, TPB, sm_x, st>>>(xin, in_map, T1, Lx, a.logL[0], a.nb[0], a.nb[1], a.nb[2],
                                       tw, twmax);
  const int R_ = a.R, Lyl = Ly / R_;
  size_t sm_yz = sizeof(cx<R>) * ((Lyl / 2 > 0 ? Lyl / 2 : 1) + (Lz / 2 > 0 ? Lz / 2 : 1) +
                                  (R_ > 1 ? Ly : 0) + (size_t)Lyl * (Lz + 1));
  dim3 gyz(Lx, R_);
  if (evs) cudaEventRecord(evs[1], st);
  if (S.is_complex) {
    k_yz<R, R, true><<<gyz, TPB, sm_yz, st>>>(T1, T4, reinterpret_cast<const R*>(S.d[prec]),
                                             a.conj, Lx, Ly, a.logL[1], Lz, a.logL[2], a.logR,
                                             a.nb[1], a.nb[2], a.na[1], a.na[2], tw, twmax);
  } else {
    k_yz<R, R, false><<<gyz, TPB, sm_yz, st>>>(T1, T4, reinterpret_cast<const R*>(S.d[prec]),
                                              0, Lx, Ly, a.logL[1], Lz, a.logL[2], a.logR,
                                              a.nb[1], a.nb[2], a.na[1], a.na[2], tw, twmax);
  }
  dim3 gi((a.na[1] + TY - 1) / TY, a.na[2]);
  if (evs) cudaEventRecord(evs[2], st);
  k_xinv<R, TY><<<gi, TPB, sm_x, st>>>(T4, yout, out_map, Lx, a.logL[0], R_, a.na[0], a.na[1],
                                       a.na[2], tw, twmax);
  if (evs) cudaEventRecord(evs[3], st);
  return 0;
}

size_t conv_smem_yz(const ConvApp& a, int prec) {
  const size_t es = prec == 0 ? sizeof(c64) : sizeof(c32);
  const int Ly = a.L[1], Lz = a.L[2], Lyl = Ly / a.R;
  return es * ((Lyl / 2 > 0 ? Lyl / 2 : 1) + (Lz / 2 > 0 ? Lz / 2 : 1) + (a.R > 1 ? Ly : 0) +
               (size_t)Lyl * (Lz + 1));
}

int conv_apply(const ConvApp& a, const Spectrum& S, const int32_t* in_map, const int32_t* out_map,
               const c64* xin, c64* yout, int prec, const void* tw64, const void* tw32, int twmax,
               cudaStream_t st, cudaEvent_t* evs) {
  if (prec == 0)
    return conv_apply_t<double>(a, S, in_map, out_map, xin, yout,
                                reinterpret_cast<const c64*>(tw64), twmax, st, evs);
  return conv_apply_t<float>(a, S, in_map, out_map, xin, yout,
                             reinterpret_cast<const c32*>(tw32), twmax, st, evs);
}

// ------------------------------------------------------------------------------------
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

__global__ void k_spec_store(const c64* __restrict__ full, void* d64, void* d32, size_t n,
                             int is_complex, double scale) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x) {
    const c64 v = full[p];
    if (is_complex) {
      reinterpret_cast<c64*>(d64)[p] = mk<double>(v.x * scale, v.y * scale);
      reinterpret_cast<c32*>(d32)[p] = mk<float>((float)(v.x * scale), (float)(v.y * scale));
    } else {
      reinterpret_cast<double*>(d64)[p] = v.x * scale;
      reinterpret_cast<float*>(d32)[p] = (float)(v.x * scale);
    }
  }
}

int spectrum_build(Spectrum& S, const double* d_row, const int M[3], const int na[3],
                   const int nb[3], const int sdim[3], const int odim[3], int symmetric,
                   const void* tw64, int twmax, cudaStream_t st) {
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
  k_spec_store<<<1184, 256, 0, st>>>(full, S.d[0], S.d[1], n, S.is_complex, 1.0 / (double)n);
  PEEC_CUDA_TRY(cudaGetLastError());
  PEEC_CUDA_TRY(cudaFreeAsync(full, st));
  return 0;
}

// host-side opt-in of the dynamic shared memory each conv kernel needs
int conv_prepare(const ConvApp& a) {
  for (int prec = 0; prec < 2; ++prec) {
    const size_t es = prec == 0 ? sizeof(c64) : sizeof(c32);
    const int Lx = a.L[0];
    size_t sm_x = es * ((Lx / 2 > 0 ? Lx / 2 : 1) + (size_t)16 * (Lx + 1));
    size_t sm_yz = conv_smem_yz(a, prec);
    if (prec == 0) {
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_xfwd<double, 16>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_x));
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_xinv<double, 16>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_x));
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_yz<double, double, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_yz));
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_yz<double, double, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_yz));
    } else {
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_xfwd<float, 16>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_x));
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_xinv<float, 16>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_x));
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_yz<float, float, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_yz));
      PEEC_CUDA_TRY(cudaFuncSetAttribute(k_yz<float, float, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_yz));
    }
  }
  return 0;
}

}  // namespace peec
