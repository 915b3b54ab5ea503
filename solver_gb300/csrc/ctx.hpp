// Internal declarations shared by the translation units of libpeec_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace peec {

int fail_cuda(cudaError_t e, const char* expr, const char* file, int line);
void set_error(const std::string& msg);

// One Toeplitz application y_out(lattice A) += K * x_in(lattice B), computed as a
// pruned circulant convolution on an Lx x Ly x Lz grid.
struct ConvApp {
  int L[3], logL[3];
  int nb[3];  // input lattice extents
  int na[3];  // output lattice extents
  int R = 1, logR = 0;    // ky split of the fused Y/Z pass
  int spec_id = -1;       // index into the spectrum table
  int conj = 0;           // use conj(S) (transposed application of a cross block)
  int in_fam = 0, out_fam = 0;   // lattice families (0..2 P faces, 3..5 Lp edges)
  // per-precision scratch: T1 = Lx x nbz x nby, T4 = R x Lx x naz x nay
  void* T1[2] = {nullptr, nullptr};
  void* T4[2] = {nullptr, nullptr};
};

struct Spectrum {
  int L[3];
  int is_complex = 0;
  void* d[2] = {nullptr, nullptr};  // [0] fp64, [1] fp32; layout (kx,ky,kz) kz fastest
};

// Launchers (fftconv.cu). prec: 0 = fp64, 1 = fp32. xin/yout are complex double.
// evs (nullable): 4 events recorded before/between/after the three kernels
int conv_apply(const ConvApp& a, const Spectrum& S, const int32_t* in_map,
               const int32_t* out_map, const c64* xin, c64* yout, int prec,
               const void* twiddles64, const void* twiddles32, int twmax, cudaStream_t st,
               cudaEvent_t* evs = nullptr);
int spectrum_build(Spectrum& S, const double* d_row, const int M[3], const int na[3],
                   const int nb[3], const int sdim[3], const int odim[3], int symmetric,
                   const void* twiddles64, int twmax, cudaStream_t st);

}  // namespace peec
