// GPU fill of the nine generating rows of the voxel Lp / P circulant blocks
// (compute_FFT_mutual_coupling_mats with QS_Rcc_FW == 1), one thread per lattice
// entry, FP64 throughout (the closed forms cancel ~R^5 terms down to ~s^6/R).
//
// Lp rows: compute_Lp_Voxels.jl:40-60 with round_ud_fft(.,14) coordinates
// (:807-815) and the volume-volume closed form integ_vol_vol_fft (:766-805).
// P rows: compute_row_P_sup.jl:1-104 with the face-face closed forms
// integ_surf_surf_para (compute_Lp_Voxels_QS.jl:695-730) and
// integ_surf_surf_ortho_P (compute_row_P_sup.jl:557-590).
// Lattice centres are recomputed from the origin with the reference's expression
// order (build_center_P_Voxels.jl:15-80, build_centers_Lp_with_air.jl:1-60).
// The suppression (far-field) tests of Integ_vol_vol_fft / Integ_sup_sup_P are
// evaluated; an entry that would take a far-field branch sets *bad, because only the
// near-field closed forms are implemented (on uniform voxels those branches need
// centre distances beyond ~200 voxel edges).
#include <math.h>
#include <math_constants.h>

#include "ctx.hpp"

namespace peec {

__device__ __forceinline__ double lgc(double v) {  // real(log(complex(v))), v >= 0
  return v > 0 ? log(v) : (v == 0 ? -INFINITY : log(fabs(v)));
}
__device__ __forceinline__ double fin(double t) { return isfinite(t) ? t : 0.0; }
__device__ __forceinline__ double round14(double v) { return rint(v * 1e14) / 1e14; }

__device__ double vol_vol(const double* x1v, const double* y1v, const double* z1v,
                          const double* x2v, const double* y2v, const double* z2v) {
  double sol = 0.0;
#pragma unroll 1
  for (int c = 0; c < 64; ++c) {
    const int c1 = (c >> 5) & 1, c2 = (c >> 4) & 1, c3 = (c >> 3) & 1, c4 = (c >> 2) & 1,
              c5 = (c >> 1) & 1, c6 = c & 1;
    const double X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2v[c5], Z = z1v[c3] - z2v[c6];
    const double X2 = X * X, Y2 = Y * Y, Z2 = Z * Z;
    const double R = sqrt(X2 + Y2 + Z2);
    const double t1 = (X2 * X2 + Y2 * Y2 + Z2 * Z2 - 3 * X2 * Y2 - 3 * Y2 * Z2 - 3 * X2 * Z2) * R / 60;
    const double t2 = fin((Y2 * Z2 / 4 - Y2 * Y2 / 24 - Z2 * Z2 / 24) * X * lgc(X + R));
    const double t3 = fin((Y2 * X2 / 4 - Y2 * Y2 / 24 - X2 * X2 / 24) * Z * lgc(Z + R));
    const double t4 = fin((Z2 * X2 / 4 - Z2 * Z2 / 24 - X2 * X2 / 24) * Y * lgc(Y + R));
    const double t5 = -fabs(X) * X2 * Y * Z / 6 * atan2(Y * Z, fabs(X) * R);
    const double t6 = -X * fabs(Y) * Y2 * Z / 6 * atan2(X * Z, fabs(Y) * R);
    const double t7 = -X * Y * fabs(Z) * Z2 / 6 * atan2(X * Y, fabs(Z) * R);
    const double s = t1 + t2 + t3 + t4 + t5 + t6 + t7;
    sol += ((c1 + c2 + c3 + c4 + c5 + c6 + 1) & 1) ? -s : s;
  }
  return sol;
}

__device__ __forceinline__ void minmax4(double a, double b, double c, double d, double& mn,
                                        double& mx) {
  a = fabs(a); b = fabs(b); c = fabs(c); d = fabs(d);
  mn = fmin(fmin(a, b), fmin(c, d));
  mx = fmax(fmax(a, b), fmax(c, d));
}

__device__ int chk_fft(double V1, double V2, double max_d, double min_R, double size_dim, double o1,
                       double o2) {
  const double e1 = 5e-3, e2 = 1e-3, e3 = 1e-3;
  const double max_oth = o1 > o2 ? o1 : o2;
  const double r = min_R + 1e-15;
  const double a = V1 * V2 * max_d / (r * r * r);
  const double f = size_dim / r;
  const double b = size_dim / max_oth;
  return ((b <= e3 || f < e1) && a < e2) ? 1 : 0;
}

// number of suppressed dimensions of Integ_vol_vol_fft (compute_Lp_Voxels.jl:86-172)
__device__ int lp_suppressed(const double* x1v, const double* y1v, const double* z1v,
                             const double* x2v, const double* y2v, const double* z2v) {
  const double e4 = 3e-1;
  const double a1 = fabs(x1v[1] - x1v[0]), b1 = fabs(y1v[1] - y1v[0]), c1 = fabs(z1v[1] - z1v[0]);
  const double a2 = fabs(x2v[1] - x2v[0]), b2 = fabs(y2v[1] - y2v[0]), c2 = fabs(z2v[1] - z2v[0]);
  const double V1 = a1 * b1 * c1, V2 = a2 * b2 * c2;
  double mnx, mxx, mny, mxy, mnz, mxz;
  minmax4(x1v[0] - x2v[0], x1v[0] - x2v[1], x1v[1] - x2v[0], x1v[1] - x2v[1], mnx, mxx);
  minmax4(y1v[0] - y2v[0], y1v[0] - y2v[1], y1v[1] - y2v[0], y1v[1] - y2v[1], mny, mxy);
  minmax4(z1v[0] - z2v[0], z1v[0] - z2v[1], z1v[1] - z2v[0], z1v[1] - z2v[1], mnz, mxz);
  const double min_R = sqrt(mnx * mnx + mny * mny + mnz * mnz);
  int s = 0;
  for (int side = 0; side < 2; ++side) {
    const double a = side ? a2 : a1, b = side ? b2 : b1, c = side ? c2 : c1;
    int sx = 0, sy = 0, sz = 0;
    if (a <= b && a <= c) {
      sx = chk_fft(V1, V2, mxx, min_R, a, b, c);
      if (sx && fmax(b, c) / (min_R + 1e-15) < e4) {
        sy = chk_fft(V1, V2, mxy, min_R, b, a, c);
        sz = chk_fft(V1, V2, mxz, min_R, c, a, b);
      }
    } else if (b <= a && b <= c) {
      sy = chk_fft(V1, V2, mxy, min_R, b, a, c);
      if (sy && fmax(a, c) / (min_R + 1e-15) < e4) {
        sx = chk_fft(V1, V2, mxx, min_R, a, b, c);
        sz = chk_fft(V1, V2, mxz, min_R, c, a, b);
      }
    } else {
      sz = chk_fft(V1, V2, mxz, min_R, c, a, b);
      if (sz && fmax(a, b) / (min_R + 1e-15) < e4) {
        sx = chk_fft(V1, V2, mxx, min_R, a, b, c);
        sy = chk_fft(V1, V2, mxy, min_R, b, a, c);
      }
    }
    s += sx + sy + sz;
  }
  return s;
}

// lattice centre of index (i,j,k); half = ceil(i/2)-style lattice per axis
__device__ __forceinline__ double ctr(double o, double s, int i, int half) {
  const double idx = half ? (double)(i >> 1) : (double)i;
  return o + s * idx + s / 2;
}

struct LpRowArgs {
  int dir;           // 0,1,2
  int M[3];          // lattice extents
  double o[3], s[3];
  double escal;
};

__device__ __forceinline__ double lp_center(const LpRowArgs& a, int axis, int i) {
  // 0.5*(A+B) of the two air-voxel centres along the edge direction
  const double A = a.o[axis] + a.s[axis] * (double)i + a.s[axis] / 2;
  if (axis != a.dir) return 0.5 * (A + A);
  const double B = a.o[axis] + a.s[axis] * (double)(i + 1) + a.s[axis] / 2;
  return 0.5 * (A + B);
}

__global__ void k_fill_lp(LpRowArgs a, double* row, int64_t N, int* bad) {
  const double sx = a.s[0], sy = a.s[1], sz = a.s[2];
  double S = sy * sz * sy * sz;
  if (a.dir == 1) S = sx * sz * sx * sz;
  else if (a.dir == 2) S = sx * sy * sx * sy;
  const double c1x = lp_center(a, 0, 0), c1y = lp_center(a, 1, 0), c1z = lp_center(a, 2, 0);
  const double x1v[2] = {round14(c1x - sx / 2), round14(c1x + sx / 2)};
  const double y1v[2] = {round14(c1y - sy / 2), round14(c1y + sy / 2)};
  const double z1v[2] = {round14(c1z - sz / 2), round14(c1z + sz / 2)};
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % a.M[0]);
    const int j = (int)((p / a.M[0]) % a.M[1]);
    const int k = (int)(p / ((int64_t)a.M[0] * a.M[1]));
    const double cx = lp_center(a, 0, i), cy = lp_center(a, 1, j), cz = lp_center(a, 2, k);
    const double x2v[2] = {round14(cx - sx / 2), round14(cx + sx / 2)};
    const double y2v[2] = {round14(cy - sy / 2), round14(cy + sy / 2)};
    const double z2v[2] = {round14(cz - sz / 2), round14(cz + sz / 2)};
    if (lp_suppressed(x1v, y1v, z1v, x2v, y2v, z2v) != 0) {
      atomicOr(bad, 1);
      row[p] = CUDART_NAN;
      continue;
    }
    const double v = vol_vol(x1v, y1v, z1v, x2v, y2v, z2v);
    row[p] = (p == 0) ? 0.0 : a.escal * (1e-7 / S * v);
  }
}

// ---------------------------------------------------------------------------------
// P rows
// ---------------------------------------------------------------------------------

__device__ double ss_para(const double* x1v, const double* y1v, double z1, const double* x2v,
                          const double* y2v, double z2) {
  double sol = 0.0;
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const int c1 = (c >> 3) & 1, c2 = (c >> 2) & 1, c3 = (c >> 1) & 1, c4 = c & 1;
    const double X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2v[c3], Z = z1 - z2;
    const double R = sqrt(X * X + Y * Y + Z * Z);
    const double t1 = -1.0 / 6 * (X * X + Y * Y - 2 * Z * Z) * R;
    const double t2 = -X * Y * fabs(Z) * atan2(X * Y, fabs(Z) * R);
    const double t3 = fin(0.5 * (X * X - Z * Z) * Y * lgc(Y + R));
    const double t4 = fin(0.5 * (Y * Y - Z * Z) * X * lgc(X + R));
    const double s = t1 + t2 + t3 + t4;
    sol += ((c1 + c2 + c3 + c4) & 1) ? -s : s;
  }
  return sol;
}

__device__ double ss_ortho(const double* x1v, const double* y1v, double z1, const double* x2v,
                           double y2, const double* z2v) {
  double sol = 0.0;
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const int c1 = (c >> 3) & 1, c2 = (c >> 2) & 1, c3 = (c >> 1) & 1, c4 = c & 1;
    const double X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2, Z = z1 - z2v[c3];
    const double R = sqrt(X * X + Y * Y + Z * Z);
    const double t1 = -1.0 / 3 * Y * Z * R;
    const double t2 = -0.5 * X * fabs(Z) * Z * atan2(X * Y, fabs(Z) * R);
    const double t3 = -0.5 * X * fabs(Y) * Y * atan2(X * Z, fabs(Y) * R);
    const double t4 = -1.0 / 6 * fabs(X) * X * X * atan2(Y * Z, fabs(X) * R);
    const double t5 = fin(X * Y * Z * lgc(X + R));
    const double t6 = fin((0.5 * X * X - 1.0 / 6 * Z * Z) * Z * lgc(Y + R));
    const double t7 = fin((0.5 * X * X - 1.0 / 6 * Y * Y) * Y * lgc(Z + R));
    const double s = t1 + t2 + t3 + t4 + t5 + t6 + t7;
    sol += ((c1 + c2 + c3 + c4) & 1) ? -s : s;
  }
  return sol;
}

__device__ int chk_pp(double S1, double S2, double max_d, double min_R, double size_dim, double o1,
                      double o2) {
  const double e1 = 5e-3, e2 = 1e-3, e3 = 1e-3, e4 = 3e-1;
  const double max_oth = o1 * o2;
  const double r = min_R + 1e-15;
  const double condS = fmax(max_oth, size_dim) / r;
  const double a = S1 * S2 * max_d / (r * r * r);
  const double f = size_dim / r;
  const double b = size_dim / max_oth;
  return (condS < e4 && (b <= e3 || f < e1) && a < e2) ? 1 : 0;
}

// Integ_sup_sup_P restricted to its surface-surface branch
__device__ double sup_sup(double xc1, double yc1, double zc1, double xc2, double yc2, double zc2,
                          double a1, double b1, double c1, double a2, double b2, double c2,
                          int* unsup) {
  const double x1v[2] = {xc1 - a1 / 2, xc1 + a1 / 2}, y1v[2] = {yc1 - b1 / 2, yc1 + b1 / 2},
               z1v[2] = {zc1 - c1 / 2, zc1 + c1 / 2};
  const double x2v[2] = {xc2 - a2 / 2, xc2 + a2 / 2}, y2v[2] = {yc2 - b2 / 2, yc2 + b2 / 2},
               z2v[2] = {zc2 - c2 / 2, zc2 + c2 / 2};
  int p1 = 2, p2 = 2;
  if (a1 <= b1 && a1 <= c1) { p1 = 0; a1 = 1; }
  else if (b1 <= a1 && b1 <= c1) { p1 = 1; b1 = 1; }
  else { c1 = 1; }
  if (a2 <= b2 && a2 <= c2) { p2 = 0; a2 = 1; }
  else if (b2 <= a2 && b2 <= c2) { p2 = 1; b2 = 1; }
  else { c2 = 1; }
  const double s1 = a1 * b1 * c1, s2 = a2 * b2 * c2;
  double mnx, mxx, mny, mxy, mnz, mxz;
  minmax4(x1v[0] - x2v[0], x1v[0] - x2v[1], x1v[1] - x2v[0], x1v[1] - x2v[1], mnx, mxx);
  minmax4(y1v[0] - y2v[0], y1v[0] - y2v[1], y1v[1] - y2v[0], y1v[1] - y2v[1], mny, mxy);
  minmax4(z1v[0] - z2v[0], z1v[0] - z2v[1], z1v[1] - z2v[0], z1v[1] - z2v[1], mnz, mxz);
  const double min_R = sqrt(mnx * mnx + mny * mny + mnz * mnz);
  int sx1 = chk_pp(s1, s2, mxx, min_R, a1, b1, c1), sx2 = chk_pp(s1, s2, mxx, min_R, a2, b2, c2);
  int sy1 = chk_pp(s1, s2, mxy, min_R, b1, a1, c1), sy2 = chk_pp(s1, s2, mxy, min_R, b2, a2, c2);
  int sz1 = chk_pp(s1, s2, mxz, min_R, c1, a1, b1), sz2 = chk_pp(s1, s2, mxz, min_R, c2, a2, b2);
  if (p1 == 0) sx1 = 1; else if (p1 == 1) sy1 = 1; else sz1 = 1;
  if (p2 == 0) sx2 = 1; else if (p2 == 1) sy2 = 1; else sz2 = 1;
  if (sx1 + sy1 + sz1 + sx2 + sy2 + sz2 != 2) {
    *unsup = 1;
    return CUDART_NAN;
  }
  if (p1 == 0) {
    if (p2 == 0) return a1 * a2 * ss_para(y1v, z1v, xc1, y2v, z2v, xc2);
    if (p2 == 1) return a1 * b2 * ss_ortho(z1v, y1v, xc1, z2v, yc2, x2v);
    return a1 * c2 * ss_ortho(y1v, z1v, xc1, y2v, zc2, x2v);
  }
  if (p1 == 1) {
    if (p2 == 0) return b1 * a2 * ss_ortho(z1v, x1v, yc1, z2v, xc2, y2v);
    if (p2 == 1) return b1 * b2 * ss_para(x1v, z1v, yc1, x2v, z2v, yc2);
    return b1 * c2 * ss_ortho(x1v, z1v, yc1, x2v, zc2, y2v);
  }
  if (p2 == 0) return c1 * a2 * ss_ortho(y1v, x1v, zc1, y2v, xc2, z2v);
  if (p2 == 1) return c1 * b2 * ss_ortho(x1v, y1v, zc1, x2v, yc2, z2v);
  return c1 * c2 * ss_para(x1v, y1v, zc1, x2v, y2v, zc2);
}

struct PRowArgs {
  int caser, caser2;
  int M[3];
  int half[3];  // interleaved axis: centre index ceil(i/2)
  double o[3], s[3];
  double escal;
};

__device__ __forceinline__ void face(int caser, double cx, double cy, double cz, double sx,
                                     double sy, double sz, double* fc, double* ext, double* d) {
  fc[0] = cx; fc[1] = cy; fc[2] = cz;
  switch (caser) {
    case 1: fc[1] = cy - sy / 2; ext[0] = sx; ext[1] = 0; ext[2] = sz; d[0] = sx; d[1] = sz; break;
    case 2: fc[1] = cy + sy / 2; ext[0] = sx; ext[1] = 0; ext[2] = sz; d[0] = sx; d[1] = sz; break;
    case 3: fc[0] = cx - sx / 2; ext[0] = 0; ext[1] = sy; ext[2] = sz; d[0] = sy; d[1] = sz; break;
    case 4: fc[0] = cx + sx / 2; ext[0] = 0; ext[1] = sy; ext[2] = sz; d[0] = sy; d[1] = sz; break;
    case 5: fc[2] = cz - sz / 2; ext[0] = sx; ext[1] = sy; ext[2] = 0; d[0] = sx; d[1] = sy; break;
    default: fc[2] = cz + sz / 2; ext[0] = sx; ext[1] = sy; ext[2] = 0; d[0] = sx; d[1] = sy; break;
  }
}

__global__ void k_fill_p(PRowArgs a, double* row, int64_t N, int* bad) {
  const double pi = 3.141592653589793;
  const double eps0 = 8.854187816997944e-12;
  const double sx = a.s[0], sy = a.s[1], sz = a.s[2];
  double f1[3], e1[3], d1[2];
  face(a.caser, ctr(a.o[0], sx, 0, a.half[0]), ctr(a.o[1], sy, 0, a.half[1]),
       ctr(a.o[2], sz, 0, a.half[2]), sx, sy, sz, f1, e1, d1);
  const double A1 = d1[0] * d1[1];
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % a.M[0]);
    const int j = (int)((p / a.M[0]) % a.M[1]);
    const int k = (int)(p / ((int64_t)a.M[0] * a.M[1]));
    double f2[3], e2[3], d2[2];
    face(a.caser2, ctr(a.o[0], sx, i, a.half[0]), ctr(a.o[1], sy, j, a.half[1]),
         ctr(a.o[2], sz, k, a.half[2]), sx, sy, sz, f2, e2, d2);
    int unsup = 0;
    const double v = sup_sup(f1[0], f1[1], f1[2], f2[0], f2[1], f2[2], e1[0], e1[1], e1[2], e2[0],
                             e2[1], e2[2], &unsup);
    if (unsup) {
      atomicOr(bad, 1);
      row[p] = CUDART_NAN;
      continue;
    }
    const double pref = 1.0 / (4 * pi * eps0 * A1 * d2[0] * d2[1]);
    row[p] = a.escal * (pref * v);
  }
}

int fill_rows_gpu(const double origin[3], double sx, double sy, double sz, double escal_Lp,
                  double escal_P, int Nx, int Ny, int Nz, double* const d_rows[9],
                  const int64_t row_len[9], int* d_bad, cudaStream_t st) {
  const int grid = 152 * 8, tpb = 128;
  const int lpM[3][3] = {{Nx - 1, Ny, Nz}, {Nx, Ny - 1, Nz}, {Nx, Ny, Nz - 1}};
  for (int d = 0; d < 3; ++d) {
    if (!d_rows[d] || row_len[d] == 0) continue;
    LpRowArgs a;
    a.dir = d;
    for (int q = 0; q < 3; ++q) {
      a.M[q] = lpM[d][q];
      a.o[q] = origin[q];
    }
    a.s[0] = sx; a.s[1] = sy; a.s[2] = sz;
    a.escal = escal_Lp;
    k_fill_lp<<<grid, tpb, 0, st>>>(a, d_rows[d], row_len[d], d_bad);
  }
  // (lattice extents, interleaved axes, caser, caser2) of the six P rows
  struct PDef { int M[3]; int half[3]; int c1, c2; };
  const PDef pd[6] = {{{Nx, Ny + 1, Nz}, {0, 0, 0}, 1, 1},
                      {{Nx + 1, Ny, Nz}, {0, 0, 0}, 3, 3},
                      {{Nx, Ny, Nz + 1}, {0, 0, 0}, 5, 5},
                      {{2 * Nx + 1, 2 * Ny + 1, Nz}, {1, 1, 0}, 3, 2},
                      {{Nx, 2 * Ny + 1, 2 * Nz + 1}, {0, 1, 1}, 5, 2},
                      {{2 * Nx + 1, Ny, 2 * Nz + 1}, {1, 0, 1}, 5, 4}};
  for (int r = 0; r < 6; ++r) {
    if (!d_rows[3 + r] || row_len[3 + r] == 0) continue;
    PRowArgs a;
    a.caser = pd[r].c1;
    a.caser2 = pd[r].c2;
    for (int q = 0; q < 3; ++q) {
      a.M[q] = pd[r].M[q];
      a.half[q] = pd[r].half[q];
      a.o[q] = origin[q];
    }
    a.s[0] = sx; a.s[1] = sy; a.s[2] = sz;
    a.escal = escal_P;
    k_fill_p<<<grid, tpb, 0, st>>>(a, d_rows[3 + r], row_len[3 + r], d_bad);
  }
  PEEC_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace peec
