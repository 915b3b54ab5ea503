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

namespace peec {

int conv_all_f32(const Family*, int, const Spectrum*, const void* const*, const c64*, c64*,
                 c64*, int64_t, const void*, int, cudaStream_t, cudaEvent_t*, const ZTune*);
int conv_all_f64(const Family*, int, const Spectrum*, const void* const*, const c64*, c64*,
                 c64*, int64_t, const void*, int, cudaStream_t, cudaEvent_t*, const ZTune*);
int conv_all_ff(const Family*, int, const Spectrum*, const void* const*, const c64*, c64*,
                c64*, int64_t, const void*, int, cudaStream_t, cudaEvent_t*, const ZTune*);

// copy W_L[e] = exp(-2 pi i e / L) for e < n from the master table of length twmax
template <typename R>
__device__ void load_tw(cx<R>* dst, const cx<R>* __restrict__ master, int twmax, int L, int n) {
  const int step = twmax / L;
  for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = master[e * step];
}

// prec: PEEC_PREC_FP64 (0), PEEC_PREC_FP32 (1), PEEC_PREC_FF (2); tw[prec] the matching
// master twiddle table
int conv_all(const Family* F, int nfam, const Spectrum* spec, const void* const* ph,
             const c64* x, c64* LpI, c64* PQ, int64_t m, int prec, const void* const* tw,
             int twmax, cudaStream_t st, cudaEvent_t* ev, const ZTune* zt) {
  if (prec == 0) return conv_all_f64(F, nfam, spec, ph, x, LpI, PQ, m, tw[0], twmax, st, ev, zt);
  if (prec == 2) return conv_all_ff(F, nfam, spec, ph, x, LpI, PQ, m, tw[2], twmax, st, ev, zt);
  return conv_all_f32(F, nfam, spec, ph, x, LpI, PQ, m, tw[1], twmax, st, ev, zt);
}

// The y/z-folded and staged FP32 z passes need whole 16-column tiles (Lx a multiple of 16, so every
// staged row is 128 bytes at a 128-byte offset), at least two radix groups along z, and
// tiles that fit three (faces) / one (edges) per shared-memory budget; the edge families
// must share one circulant grid to share a launch.
static bool staged_grid(const Family& f, int zmin) {
  return f.L[0] >= 16 && f.L[0] % 16 == 0 && f.L[2] >= zmin && f.L[2] <= 128 &&
         f.dims[2] >= 1 && f.dims[2] <= f.L[2];
}

bool zpass_yz_faces(const Family* F, int nfam) {
  if (nfam < 3) return false;
  for (int f = 0; f < 3; ++f)
    if (!F[f].active || !staged_grid(F[f], 16)) return false;
  return true;
}

bool zpass_yz_edges(const Family* F, int nfam) {
  const Family* f0 = nullptr;
  for (int f = 3; f < nfam; ++f) {
    if (!F[f].active) continue;
    if (!staged_grid(F[f], 32)) return false;
    if (!f0) f0 = &F[f];
    else if (F[f].L[0] != f0->L[0] || F[f].L[1] != f0->L[1] || F[f].L[2] != f0->L[2])
      return false;
  }
  return f0 != nullptr;
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

// full (x,y,z; z fastest, DIF bit-reversed positions along each axis) -> octant R of the
// half-sample-shift form (see Spectrum), scaled, FP64
__global__ void k_spec_octant(const c64* __restrict__ full, double* o64, int Lx, int Ly, int Lz,
                              int cx, int cy, int cz, double scale) {
  const int ox = Lx / 2 + 1, oy = Ly / 2 + 1, oz = Lz / 2 + 1;
  const int nx = ilog2(Lx), ny = ilog2(Ly), nz = ilog2(Lz);
  const size_t n = (size_t)ox * oy * oz;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < n;
       o += (size_t)gridDim.x * blockDim.x) {
    const int fx = (int)(o % ox);
    const size_t rr = o / ox;
    const int fz = (int)(rr % oz), fy = (int)(rr / oz);
    const int px = brev(fx & (Lx - 1), nx), py = brev(fy & (Ly - 1), ny),
              pz = brev(fz & (Lz - 1), nz);
    const c64 v = full[((size_t)px * Ly + py) * Lz + pz];
    // R = Re(S * prod exp(+i*pi*c*f/L)); the phase angle sum is exact in double
    double ph = 0.0;
    if (cx) ph += (double)cx * fx / Lx;
    if (cy) ph += (double)cy * fy / Ly;
    if (cz) ph += (double)cz * fz / Lz;
    double sn, cs;
    sincospi(ph, &sn, &cs);
    o64[o] = (v.x * cs - v.y * sn) * scale;
  }
}

// octant R (FP64, (fy, fz, fx)) -> y/z-folded FP32 R ((fy, fz, px), px every DIF x position)
__global__ void k_spec_yzfold(const double* __restrict__ o64, float* y32, int Lx, int Ly,
                              int Lz) {
  const int ox = Lx / 2 + 1, oy = Ly / 2 + 1, oz = Lz / 2 + 1;
  const int nx = ilog2(Lx);
  const size_t n = (size_t)Lx * oy * oz;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < n;
       o += (size_t)gridDim.x * blockDim.x) {
    const int px = (int)(o % Lx);
    const size_t rr = o / Lx;  // fy * oz + fz
    int k = brev(px, nx);
    const int fx = k <= Lx / 2 ? k : Lx - k;
    y32[o] = (float)o64[rr * ox + fx];
  }
}

// phase tables of the shifted axes: E[p] = exp(-i*pi*k/L) for the signed frequency k of
// DIF position p (k = brev(p) folded into (-L/2, L/2]), FP64 and its FP32 rounding
__global__ void k_phase_table(int L, c64* e64, c32* e32) {
  const int n = ilog2(L);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < L; p += gridDim.x * blockDim.x) {
    int k = brev(p, n);
    if (k > L / 2) k -= L;
    double sn, cs;
    sincospi(-(double)k / L, &sn, &cs);
    e64[p] = mk<double>(cs, sn);
    e32[p] = mk<float>((float)cs, (float)sn);
  }
}

int phase_tables(const int L[3], void* e64[3], void* e32[3], cudaStream_t st) {
  for (int a = 0; a < 3; ++a) {
    if (e64[a]) cudaFree(e64[a]);
    if (e32[a]) cudaFree(e32[a]);
    e64[a] = e32[a] = nullptr;
    PEEC_CUDA_TRY(cudaMalloc(&e64[a], sizeof(c64) * L[a]));
    PEEC_CUDA_TRY(cudaMalloc(&e32[a], sizeof(c32) * L[a]));
    k_phase_table<<<(L[a] + 255) / 256, 256, 0, st>>>(L[a], (c64*)e64[a], (c32*)e32[a]);
  }
  PEEC_CUDA_TRY(cudaGetLastError());
  return 0;
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
  // half-sample shift per axis: |2e + o| is even about e = -o/2 (the embedding window is
  // symmetric about the same point because na - nb = -o there)
  for (int a = 0; a < 3; ++a) S.c[a] = (!symmetric && sdim[a] == 2) ? -odim[a] : 0;
  S.is_complex = symmetric ? 0 : 1;
  const size_t es64 = S.is_complex ? sizeof(c64) : sizeof(double);
  const size_t es32 = S.is_complex ? sizeof(c32) : sizeof(float);
  if (!S.d[0]) PEEC_CUDA_TRY(cudaMalloc(&S.d[0], n * es64));
  if (!S.d[1]) PEEC_CUDA_TRY(cudaMalloc(&S.d[1], n * es32));
  k_spec_store<<<1184, 256, 0, st>>>(full, S.d[0], S.d[1], S.L[0], S.L[1], S.L[2], S.is_complex,
                                     1.0 / (double)n);
  const size_t no = (size_t)(S.L[0] / 2 + 1) * (S.L[1] / 2 + 1) * (S.L[2] / 2 + 1);
  if (!S.oct) PEEC_CUDA_TRY(cudaMalloc(&S.oct, no * sizeof(double)));
  k_spec_octant<<<1184, 256, 0, st>>>(full, (double*)S.oct, S.L[0], S.L[1], S.L[2], S.c[0],
                                      S.c[1], S.c[2], 1.0 / (double)n);
  const size_t ny32 = (size_t)S.L[0] * (S.L[1] / 2 + 1) * (S.L[2] / 2 + 1);
  if (!S.yz32) PEEC_CUDA_TRY(cudaMalloc(&S.yz32, ny32 * sizeof(float)));
  k_spec_yzfold<<<1184, 256, 0, st>>>((const double*)S.oct, (float*)S.yz32, S.L[0], S.L[1],
                                      S.L[2]);
  PEEC_CUDA_TRY(cudaGetLastError());
  PEEC_CUDA_TRY(cudaFreeAsync(full, st));
  return 0;
}

}  // namespace peec
