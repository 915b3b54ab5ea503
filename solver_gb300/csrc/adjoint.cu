// Reciprocity gradient of a port voltage in per-voxel parameters (peec_adjoint): a
// scatter of the edge-current squares weighted by the edge-impedance derivatives onto
// the voxels of each edge. One thread per edge, double atomics per voxel (an edge joins
// two voxels; a voxel has at most six edges per direction pair). The atomics make the
// order of each voxel's sum vary between runs: results agree to a few ulps, not bitwise.
#include "ctx.hpp"

namespace peec {

__global__ void k_adjoint(const c64* __restrict__ x, const int32_t* __restrict__ v1,
                          const int32_t* __restrict__ v2, const c64* __restrict__ d1,
                          const c64* __restrict__ d2, double scale, int64_t m, int64_t nvox,
                          double* g) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const c64 I = x[e];
    const c64 I2 = mk<double>(I.x * I.x - I.y * I.y, 2.0 * I.x * I.y);
    const int32_t a = v1[e], b = v2[e];
    if (a >= 0 && a < nvox) {
      const c64 d = d1[e];
      atomicAdd(g + 2 * (int64_t)a, scale * (d.x * I2.x - d.y * I2.y));
      atomicAdd(g + 2 * (int64_t)a + 1, scale * (d.x * I2.y + d.y * I2.x));
    }
    if (b >= 0 && b < nvox) {
      const c64 d = d2[e];
      atomicAdd(g + 2 * (int64_t)b, scale * (d.x * I2.x - d.y * I2.y));
      atomicAdd(g + 2 * (int64_t)b + 1, scale * (d.x * I2.y + d.y * I2.x));
    }
  }
}

void launch_adjoint(const c64* x, const int32_t* v1, const int32_t* v2, const c64* d1,
                    const c64* d2, double scale, int64_t m, int64_t nvox, double* g,
                    cudaStream_t st) {
  const int grid = (int)std::min<int64_t>((m + 255) / 256, 152 * 16);
  if (m > 0) k_adjoint<<<grid > 0 ? grid : 1, 256, 0, st>>>(x, v1, v2, d1, d2, scale, m, nvox, g);
}

}  // namespace peec
