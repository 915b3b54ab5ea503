// GPU fill of the nine generating rows of the voxel Lp / P circulant blocks
// (compute_FFT_mutual_coupling_mats with QS_Rcc_FW == 1), one thread per lattice
// entry, FP64 throughout (the near-field closed forms cancel ~R^5 terms down to ~s^6/R).
//
// Lp rows: compute_Lp_Voxels.jl:40-60 with round_ud_fft(.,14) coordinates (:807-815) and
// the Integ_vol_vol_fft dispatch (:65-435): the volume-volume closed form
// integ_vol_vol_fft (:766-805) in the near field, and once a dimension passes its
// suppression test (check_condition_fft, :437-447; on uniform voxels a centre distance
// beyond ~200 edges of that dimension) the closed form of the bodies left when that
// dimension collapses (volume-surface ... point-point, :449-764).
// P rows: compute_row_P_sup.jl:1-104 with the Integ_sup_sup_P dispatch (:106-381), its
// face-face closed forms integ_surf_surf_para (compute_Lp_Voxels_QS.jl:695-730) and
// integ_surf_surf_ortho_P (:557-590), and its far-field primitives (:396-556).
//
// The far-field primitives keep the reference's arithmetic exactly (expression order,
// the zeroing of non-finite log terms, the 1e-8 nudges of integ_line_point and the
// origin-dependent collinear-line forms integ_line_line_sp_fft / _P), and this file is
// compiled without FMA contraction, so that degenerate corners (X + R rounding to 0)
// fall the same way as in the reference's scalar Float64 code.
//
// The dispatch is written over axis-indexed boxes: for each pair of bodies the
// collapsed dimensions select a primitive, whose arguments are the boxes' intervals and
// centres permuted the way the reference's case tree passes them.
// Lattice centres are recomputed from the origin with the reference's expression
// order (build_center_P_Voxels.jl:15-80, build_centers_Lp_with_air.jl:1-60).
#include <math.h>

#include <algorithm>
#include <math_constants.h>

#include "ctx.hpp"

namespace peec {

__device__ __forceinline__ double lgc(double v) {  // real(log(complex(v)))
  return v > 0 ? log(v) : (v == 0 ? -INFINITY : log(fabs(v)));
}
__device__ __forceinline__ double fin(double t) { return isfinite(t) ? t : 0.0; }
__device__ __forceinline__ double round14(double v) { return rint(v * 1e14) / 1e14; }
// (-1)^k
__device__ __forceinline__ double sgn(int k) { return (k & 1) ? -1.0 : 1.0; }

// ---------------------------------------------------------------------------------
// closed forms; corner signs are the reference's (-1)^(c1+..+cn [+1]) with 1-based c,
// i.e. (-1)^(sum0 + n [+1]) with the 0-based corner bits used here
// ---------------------------------------------------------------------------------

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
    sol += sgn(c1 + c2 + c3 + c4 + c5 + c6 + 1) * (t1 + t2 + t3 + t4 + t5 + t6 + t7);
  }
  return sol;
}

// surfaces in (x, y) planes at heights z1, z2
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
    sol += sgn(c1 + c2 + c3 + c4) * (t1 + t2 + t3 + t4);
  }
  return sol;
}

// surface in the (x, y) plane at z1 against one in the (x, z) plane at y2; pform selects
// the seven-term integ_surf_surf_ortho_P over the four-term integ_surf_surf_ortho_fft
__device__ double ss_ortho(const double* x1v, const double* y1v, double z1, const double* x2v,
                           double y2, const double* z2v, int pform) {
  double sol = 0.0;
#pragma unroll 1
  for (int c = 0; c < 16; ++c) {
    const int c1 = (c >> 3) & 1, c2 = (c >> 2) & 1, c3 = (c >> 1) & 1, c4 = c & 1;
    const double X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2, Z = z1 - z2v[c3];
    const double R = sqrt(X * X + Y * Y + Z * Z);
    const double t1 = -1.0 / 3 * Y * Z * R;
    const double t2 = -0.5 * X * fabs(Z) * Z * atan2(X * Y, fabs(Z) * R);
    double s;
    if (pform) {
      const double t3 = -0.5 * X * fabs(Y) * Y * atan2(X * Z, fabs(Y) * R);
      const double t4 = -1.0 / 6 * fabs(X) * X * X * atan2(Y * Z, fabs(X) * R);
      const double t5 = fin(X * Y * Z * lgc(X + R));
      const double t6 = fin((0.5 * X * X - 1.0 / 6 * Z * Z) * Z * lgc(Y + R));
      const double t7 = fin((0.5 * X * X - 1.0 / 6 * Y * Y) * Y * lgc(Z + R));
      s = t1 + t2 + t3 + t4 + t5 + t6 + t7;
    } else {
      const double t3 = fin(0.5 * (X * X - Z * Z) * Y * lgc(Y + R));
      const double t4 = fin(0.5 * (X * X - Y * Y) * X * lgc(X + R));
      s = t1 + t2 + t3 + t4;
    }
    sol += sgn(c1 + c2 + c3 + c4) * s;
  }
  return sol;
}

// line [xv] at (y3, z3) against the point (x1, y1, z1)
__device__ double line_point(const double* xv, double y3, double z3, double x1, double y1,
                             double z1) {
  const double x3 = xv[0], x4 = xv[1];
  double chk = 1.0 / (x1 - x3);
  if (isnan(chk) || isinf(chk)) x1 = x1 - 1e-8;
  chk = 1.0 / (x1 - x4);
  if (isnan(chk) || (isinf(chk) && x1 > 0)) x1 = x1 + 1e-8;
  const double R1 = sqrt((x1 - x3) * (x1 - x3) + (y1 - y3) * (y1 - y3) + (z1 - z3) * (z1 - z3));
  const double R2 = sqrt((x1 - x4) * (x1 - x4) + (y1 - y3) * (y1 - y3) + (z1 - z3) * (z1 - z3));
  double Ip = log((x1 - x3) + R1) - log((x1 - x4) + R2);
  if (!isfinite(Ip))
    Ip = (x1 - x3) / fabs(x1 - x3) * log(fabs(x1 - x3)) -
         (x1 - x4) / fabs(x1 - x4) * log(fabs(x1 - x4));
  return Ip;
}

// point (x1, y1, z1) against the surface [x2v] x [y2v] at height z2; pform 3 (the dense
// RIS Lp tree, integ_point_sup_sharedRis, Song_improved_Ivana_strategy.jl:449-478) takes
// the arctangent of the quotient, NaN where both of its parts vanish
__device__ double point_sup(double x1, double y1, double z1, const double* x2v, const double* y2v,
                            double z2, int pform) {
  double sol = 0.0;
  for (int c = 0; c < 4; ++c) {
    const int c1 = c >> 1, c2 = c & 1;
    const double X = x1 - x2v[c1], Y = y1 - y2v[c2], Z = z1 - z2;
    const double R = sqrt(X * X + Y * Y + Z * Z);
    const double t3 = pform == 3 ? -fabs(Z) * atan(X * Y / (fabs(Z) * R))
                                 : -fabs(Z) * atan2(X * Y, fabs(Z) * R);
    sol += sgn(c1 + c2) * (fin(X * lgc(Y + R)) + fin(Y * lgc(X + R)) + t3);
  }
  return sol;
}

// collinear lines, in absolute coordinates as the reference writes them
__device__ double ll_sp(const double* x1v, const double* x2v, int pform) {
  double sol = 0.0;
  for (int c = 0; c < 4; ++c) {
    const int c1 = c >> 1, c2 = c & 1;
    const double x1 = x1v[c1], x2 = x2v[c2];
    const double R = sqrt((x1 - x2) * (x1 - x2));
    double t;
    if (pform >= 2)  // integ_line_line_sp of compute_Lp_Voxels_QS.jl:501-520 and the dense
                     // RIS forms (Song_improved_Ivana_strategy.jl:510-532,
                     // Song_P_improved_Ivana_strategy.jl:360-382)
      t = (x1 - x2) / R * (x1 - x2 * lgc(x2 - x1) + x1 * lgc(x1 - x2));
    else {
      t = (x1 - x2) / R * (x1 - x2 * lgc(x2 - x1));
      if (pform) t = t + x1 * lgc(x1 - x2);
    }
    sol += sgn(c1 + c2 + 1) * fin(t);
  }
  return sol;
}

// parallel lines along x at (y1, z1) and (y2, z2)
__device__ double ll_parall(const double* x1v, double y1, double z1, const double* x2v, double y2,
                            double z2, int pform) {
  const double dy = y1 - y2, dz = z1 - z2;
  if (fabs(dy) < 1e-10 && fabs(dz) < 1e-10) return ll_sp(x1v, x2v, pform);
  double sol = 0.0;
  for (int c = 0; c < 4; ++c) {
    const int c1 = c >> 1, c2 = c & 1;
    const double X = x1v[c1] - x2v[c2];
    const double R = sqrt(X * X + dy * dy + dz * dz);
    sol += sgn(c1 + c2 + 1) * (fin(X * lgc(X + R)) - R);
  }
  return sol;
}

// line along x at (y1, z1) against a line along y at (x2, z2)
__device__ double ll_ortho(const double* x1v, double y1, double z1, double x2, const double* y2v,
                           double z2) {
  double sol = 0.0;
  for (int c = 0; c < 4; ++c) {
    const int c1 = c >> 1, c2 = c & 1;
    const double X = x1v[c1] - x2, Y = y1 - y2v[c2], Z = z1 - z2;
    const double R = sqrt(X * X + Y * Y + Z * Z);
    sol += sgn(c1 + c2 + 1) *
           (fin(X * lgc(Y + R)) + fin(Y * lgc(X + R)) - fabs(Z) * atan2(X * Y, fabs(Z) * R));
  }
  return sol;
}

// the triple antiderivative of 1/R (six terms)
__device__ double f111(double X, double Y, double Z) {
  const double R = sqrt(X * X + Y * Y + Z * Z);
  const double t1 = fin(Y * Z * lgc(X + R));
  const double t2 = fin(X * Z * lgc(Y + R));
  const double t3 = fin(Y * X * lgc(Z + R));
  const double t4 = -0.5 * fabs(Z) * Z * atan2(X * Y, fabs(Z) * R);
  const double t5 = -0.5 * fabs(Y) * Y * atan2(X * Z, fabs(Y) * R);
  const double t6 = -0.5 * fabs(X) * X * atan2(Y * Z, fabs(X) * R);
  return t1 + t2 + t3 + t4 + t5 + t6;
}

__device__ double point_vol(double x1, double y1, double z1, const double* x2v, const double* y2v,
                            const double* z2v) {
  double sol = 0.0;
  for (int c = 0; c < 8; ++c) {
    const int c1 = c >> 2, c2 = (c >> 1) & 1, c3 = c & 1;
    sol += sgn(c1 + c2 + c3) * f111(x1 - x2v[c1], y1 - y2v[c2], z1 - z2v[c3]);
  }
  return sol;
}

// line along x at (y1, z1) against the surface [y2v] x [z2v] at x2; pform selects the
// six-term integ_line_surf_ortho_P over the three-term integ_line_surf_ortho_fft
__device__ double ls_ortho(const double* x1v, double y1, double z1, double x2, const double* y2v,
                           const double* z2v, int pform) {
  double sol = 0.0;
  for (int c = 0; c < 8; ++c) {
    const int c1 = c >> 2, c2 = (c >> 1) & 1, c3 = c & 1;
    const double X = x1v[c1] - x2, Y = y1 - y2v[c2], Z = z1 - z2v[c3];
    double v;
    if (pform) {
      v = f111(X, Y, Z);
    } else {
      const double R = sqrt(X * X + Y * Y + Z * Z);
      v = fin(Y * Z * lgc(X + R)) + fin(X * Z * lgc(Y + R)) - fabs(Z) * atan2(X * Y, fabs(Z) * R);
    }
    sol += sgn(c1 + c2 + c3 + 1) * v;
  }
  return sol;
}

// surface [x1v] x [y1v] at z1 against a line along x at (y2, z2)
__device__ double ls_para(const double* x1v, const double* y1v, double z1, const double* x2v,
                          double y2, double z2) {
  double sol = 0.0;
  for (int c = 0; c < 8; ++c) {
    const int c1 = c >> 2, c2 = (c >> 1) & 1, c3 = c & 1;
    const double X = x1v[c1] - x2v[c3], Y = y1v[c2] - y2, Z = z1 - z2;
    const double R = sqrt(X * X + Y * Y + Z * Z);
    const double t1 = fin(X * Y * lgc(X + R));
    const double t2 = fin((X * X - Z * Z) / 2 * lgc(Y + R));
    const double t3 = -X * fabs(Z) * atan2(X * Y, fabs(Z) * R);
    const double t4 = -Y / 2 * R;
    sol += sgn(c1 + c2 + c3) * (t1 + t2 + t3 + t4);
  }
  return sol;
}

// volume against a line along x at (y2, z2)
__device__ double line_vol(const double* x1v, const double* y1v, const double* z1v,
                           const double* x2v, double y2, double z2) {
  double sol = 0.0;
#pragma unroll 1
  for (int c = 0; c < 16; ++c) {
    const int c1 = c >> 3, c2 = (c >> 2) & 1, c3 = (c >> 1) & 1, c4 = c & 1;
    const double X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2, Z = z1v[c3] - z2;
    const double R = sqrt(X * X + Y * Y + Z * Z);
    const double aX = fabs(X);
    const double t1 = -1.0 / 3 * Y * Z * R;
    const double t2 = -0.5 * X * fabs(Z) * Z * atan2(X * Y, fabs(Z) * R);
    const double t3 = -0.5 * X * fabs(Y) * Y * atan2(X * Z, fabs(Y) * R);
    const double t4 = -1.0 / 6 * (aX * aX * aX) * atan2(Y * Z, aX * R);
    const double t5 = fin(X * Y * Z * lgc(X + R));
    const double t6 = fin((0.5 * (X * X) - 1.0 / 6 * (Z * Z)) * Z * lgc(Y + R));
    const double t7 = fin((0.5 * (X * X) - 1.0 / 6 * (Y * Y)) * Y * lgc(Z + R));
    sol += sgn(c1 + c2 + c3 + c4 + 1) * (t1 + t2 + t3 + t4 + t5 + t6 + t7);
  }
  return sol;
}

// volume against the surface [x2v] x [y2v] at z2; pform 2: integ_vol_surf of
// compute_Lp_Voxels_QS.jl:777-824, whose second and third terms carry a factor (z1 - z2)
__device__ double vol_surf(const double* x1v, const double* y1v, const double* z1v,
                           const double* x2v, const double* y2v, double z2, int pform) {
  double sol = 0.0;
#pragma unroll 1
  for (int c = 0; c < 32; ++c) {
    const int c1 = c >> 4, c2 = (c >> 3) & 1, c3 = (c >> 2) & 1, c4 = (c >> 1) & 1, c5 = c & 1;
    const double X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2v[c5], Z = z1v[c3] - z2;
    const double X2 = X * X, Y2 = Y * Y, Z2 = Z * Z;
    const double R = sqrt(X2 + Y2 + Z2);
    const double aX = fabs(X), aY = fabs(Y);
    const double t1 = (Z2 / 12 - (X2 + Y2) / 8) * Z * R;
    const double t2 = (pform == 2 || pform == 3) ? fin((Y2 / 2 - Z2 / 6) * X * Z * lgc(X + R))
                                 : fin((Y2 / 2 - Z2 / 6) * X * lgc(X + R));
    const double t3 = (pform == 2 || pform == 3) ? fin((X2 / 2 - Z2 / 6) * Y * Z * lgc(Y + R))
                                 : fin((X2 / 2 - Z2 / 6) * Y * lgc(Y + R));
    const double t4 = fin((-(X2 * X2) / 24 - (Y2 * Y2) / 24 + (Y2 * X2) / 4) * lgc(Z + R));
    const double t5 = -(aX * aX * aX) * Y / 6 * atan2(Y * Z, aX * R);
    const double t6 = -X * (aY * aY * aY) / 6 * atan2(X * Z, aY * R);
    const double t7 = -X * Y * fabs(Z) * Z / 2 * atan2(X * Y, fabs(Z) * R);
    sol += sgn(c1 + c2 + c3 + c4 + c5 + 1) * (t1 + t2 + t3 + t4 + t5 + t6 + t7);
  }
  return sol;
}

// ---------------------------------------------------------------------------------
// dispatch over axis-indexed boxes
// ---------------------------------------------------------------------------------

struct Box {
  double iv[3][2];  // interval per axis
  double c[3];      // centre per axis
  double len[3];    // edge length per axis (1 for a face normal in the P tree)
  int s[3];         // dimension collapsed
  int n;            // number collapsed
};

// the two axes other than a, in increasing order
__device__ __forceinline__ void others(int a, int& u, int& v) {
  u = a == 0 ? 1 : 0;
  v = a == 2 ? 1 : 2;
}
__device__ __forceinline__ int open_axis(const Box& b) { return !b.s[0] ? 0 : (!b.s[1] ? 1 : 2); }
__device__ __forceinline__ int shut_axis(const Box& b) { return b.s[0] ? 0 : (b.s[1] ? 1 : 2); }

// The integral of 1/R over the two boxes with their collapsed dimensions, each collapsed
// length entering as a factor (the shared case tree of Integ_vol_vol_fft,
// Integ_sup_sup_P and the Rcc path's Integ_vol_vol; pform 1 selects the _P primitives,
// pform 2 those of compute_Lp_Voxels_QS.jl). In the Rcc tree's orthogonal surface-surface
// case the reference calls integ_surf_surf_ortho with an interval where it takes a
// coordinate (compute_Lp_Voxels_QS.jl:330-352), which Julia cannot apply: NaN here, which
// the row kernel reports. pform 3 is the dense RIS Lp tree (Song_improved_Ivana_strategy2,
// Song_improved_Ivana_strategy.jl:1-404): the pform 2 primitives with the seven-term
// orthogonal surface-surface form and the quotient arctangent of the point-surface form.
// pform 4 is the dense RIS P tree (Song_P_improved_Ivana_strategy.jl:1-256): the _P
// primitives with the collinear-line form of pform 2.
__device__ __noinline__ double integ_boxes(const Box& A, const Box& B, int pform) {
  const double V1 = A.len[0] * A.len[1] * A.len[2], V2 = B.len[0] * B.len[1] * B.len[2];
  switch (A.n + B.n) {
    case 6: {
      const double dx = A.c[0] - B.c[0], dy = A.c[1] - B.c[1], dz = A.c[2] - B.c[2];
      return V1 * V2 / sqrt(dx * dx + dy * dy + dz * dz);
    }
    case 5: {  // point - line
      const Box& L = A.n == 3 ? B : A;
      const Box& P = A.n == 3 ? A : B;
      const int i = open_axis(L);
      int j, k;
      others(i, j, k);
      return V1 * V2 / L.len[i] * line_point(L.iv[i], L.c[j], L.c[k], P.c[i], P.c[j], P.c[k]);
    }
    case 4: {
      if (A.n == 3 || B.n == 3) {  // point - surface
        const Box& P = A.n == 3 ? A : B;
        const Box& S = A.n == 3 ? B : A;
        const int nrm = shut_axis(S);
        const int u = nrm == 0 ? 2 : 0, v = nrm == 1 ? 2 : 1;
        const double Vp = A.n == 3 ? V1 : V2;
        return Vp * S.len[nrm] *
               point_sup(P.c[u], P.c[v], P.c[nrm], S.iv[u], S.iv[v], S.c[nrm], pform);
      }
      // line - line
      const int i = open_axis(A), j = open_axis(B);
      int o1, o2, q1, q2;
      others(i, o1, o2);
      others(j, q1, q2);
      const double w = A.len[o1] * A.len[o2] * B.len[q1] * B.len[q2];
      if (i == j) return w * ll_parall(A.iv[i], A.c[o1], A.c[o2], B.iv[i], B.c[o1], B.c[o2], pform);
      const int k = 3 - i - j;
      return w * ll_ortho(A.iv[i], A.c[j], A.c[k], B.c[i], B.iv[j], B.c[k]);
    }
    case 3: {
      if (A.n == 3)
        return A.len[0] * A.len[1] * A.len[2] * point_vol(A.c[0], A.c[1], A.c[2], B.iv[0], B.iv[1], B.iv[2]);
      if (B.n == 3)
        return B.len[0] * B.len[1] * B.len[2] * point_vol(B.c[0], B.c[1], B.c[2], A.iv[0], A.iv[1], A.iv[2]);
      // surface - line
      const Box& S = A.n == 1 ? A : B;
      const Box& L = A.n == 1 ? B : A;
      const int nrm = shut_axis(S), i = open_axis(L);
      int q1, q2;
      others(i, q1, q2);
      const double w = S.len[nrm] * L.len[q1] * L.len[q2];
      if (i == nrm) {
        int u, v;
        others(i, u, v);
        return w * ls_ortho(L.iv[i], L.c[u], L.c[v], S.c[nrm], S.iv[u], S.iv[v], pform);
      }
      const int m = 3 - i - nrm;
      return w * ls_para(S.iv[i], S.iv[m], S.c[nrm], L.iv[i], L.c[m], L.c[nrm]);
    }
    case 2: {
      if (A.n == 2 || B.n == 2) {  // line - volume
        const Box& L = A.n == 2 ? A : B;
        const Box& V = A.n == 2 ? B : A;
        const int i = open_axis(L);
        int o1, o2;
        others(i, o1, o2);
        return L.len[o1] * L.len[o2] *
               line_vol(V.iv[i], V.iv[o1], V.iv[o2], L.iv[i], L.c[o1], L.c[o2]);
      }
      // surface - surface
      const int n1 = shut_axis(A), n2 = shut_axis(B);
      const double w = A.len[n1] * B.len[n2];
      if (n1 == n2) {
        int u, v;
        others(n1, u, v);
        return w * ss_para(A.iv[u], A.iv[v], A.c[n1], B.iv[u], B.iv[v], B.c[n1]);
      }
      if (pform == 2) return nan("");
      const int a = 3 - n1 - n2;
      return w * ss_ortho(A.iv[a], A.iv[n2], A.c[n1], B.iv[a], B.c[n2], B.iv[n1], pform);
    }
    case 1: {  // surface - volume
      const Box& S = A.n == 1 ? A : B;
      const Box& V = A.n == 1 ? B : A;
      const int nrm = shut_axis(S);
      int u, v;
      others(nrm, u, v);
      return S.len[nrm] * vol_surf(V.iv[u], V.iv[v], V.iv[nrm], S.iv[u], S.iv[v], S.c[nrm], pform);
    }
    default:
      return vol_vol(A.iv[0], A.iv[1], A.iv[2], B.iv[0], B.iv[1], B.iv[2]);
  }
}

__device__ __forceinline__ void minmax4(double a, double b, double c, double d, double& mn,
                                        double& mx) {
  a = fabs(a); b = fabs(b); c = fabs(c); d = fabs(d);
  mn = fmin(fmin(a, b), fmin(c, d));
  mx = fmax(fmax(a, b), fmax(c, d));
}

// closest-corner distance of the two boxes and the largest corner offset per axis
__device__ __forceinline__ double box_gaps(const Box& A, const Box& B, double mxd[3]) {
  double mn[3];
  for (int d = 0; d < 3; ++d)
    minmax4(A.iv[d][0] - B.iv[d][0], A.iv[d][0] - B.iv[d][1], A.iv[d][1] - B.iv[d][0],
            A.iv[d][1] - B.iv[d][1], mn[d], mxd[d]);
  return sqrt(mn[0] * mn[0] + mn[1] * mn[1] + mn[2] * mn[2]);
}

// check_condition_fft (compute_Lp_Voxels.jl:437-447)
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

// suppression flags of Integ_vol_vol_fft (compute_Lp_Voxels.jl:86-172): the smallest
// edge first, the other two only when the larger of them is under 0.3 min_R
__device__ void lp_flags(Box& A, Box& B) {
  const double e4 = 3e-1;
  double mxd[3];
  const double min_R = box_gaps(A, B, mxd);
  const double V1 = A.len[0] * A.len[1] * A.len[2], V2 = B.len[0] * B.len[1] * B.len[2];
  for (int side = 0; side < 2; ++side) {
    Box& X = side ? B : A;
    const double* l = X.len;
    const int first = (l[0] <= l[1] && l[0] <= l[2]) ? 0 : ((l[1] <= l[0] && l[1] <= l[2]) ? 1 : 2);
    int u, v;
    others(first, u, v);
    X.s[0] = X.s[1] = X.s[2] = 0;
    X.s[first] = chk_fft(V1, V2, mxd[first], min_R, l[first], l[u], l[v]);
    if (X.s[first] && fmax(l[u], l[v]) / (min_R + 1e-15) < e4) {
      int a, b;
      others(u, a, b);
      X.s[u] = chk_fft(V1, V2, mxd[u], min_R, l[u], l[a], l[b]);
      others(v, a, b);
      X.s[v] = chk_fft(V1, V2, mxd[v], min_R, l[v], l[a], l[b]);
    }
    X.n = X.s[0] + X.s[1] + X.s[2];
  }
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
  int form;          // 0: Integ_vol_vol_fft (QS fill); 2: Integ_vol_vol (Rcc rows)
};

__device__ __forceinline__ double lp_center(const LpRowArgs& a, int axis, int i) {
  // 0.5*(A+B) of the two air-voxel centres along the edge direction
  const double A = a.o[axis] + a.s[axis] * (double)i + a.s[axis] / 2;
  if (axis != a.dir) return 0.5 * (A + A);
  const double B = a.o[axis] + a.s[axis] * (double)(i + 1) + a.s[axis] / 2;
  return 0.5 * (A + B);
}

// voxel box of compute_Lp_Voxels: round_ud_fft(centre -+ s/2, 14) per axis
__device__ __forceinline__ void lp_box(Box& b, const double c[3], const double s[3]) {
  for (int d = 0; d < 3; ++d) {
    b.iv[d][0] = round14(c[d] - s[d] / 2);
    b.iv[d][1] = round14(c[d] + s[d] / 2);
    b.c[d] = 0.5 * (b.iv[d][0] + b.iv[d][1]);
    b.len[d] = fabs(b.iv[d][1] - b.iv[d][0]);
  }
}

__global__ void k_fill_lp(LpRowArgs a, double* row, int64_t N, int* bad) {
  const double sx = a.s[0], sy = a.s[1], sz = a.s[2];
  double S = sy * sz * sy * sz;
  if (a.dir == 1) S = sx * sz * sx * sz;
  else if (a.dir == 2) S = sx * sy * sx * sy;
  const double c1[3] = {lp_center(a, 0, 0), lp_center(a, 1, 0), lp_center(a, 2, 0)};
  Box A;
  lp_box(A, c1, a.s);
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % a.M[0]);
    const int j = (int)((p / a.M[0]) % a.M[1]);
    const int k = (int)(p / ((int64_t)a.M[0] * a.M[1]));
    const double c2[3] = {lp_center(a, 0, i), lp_center(a, 1, j), lp_center(a, 2, k)};
    Box B;
    lp_box(B, c2, a.s);
    lp_flags(A, B);
    const double v = (A.n + B.n == 0)
                         ? vol_vol(A.iv[0], A.iv[1], A.iv[2], B.iv[0], B.iv[1], B.iv[2])
                         : integ_boxes(A, B, a.form);
    const double e = (p == 0) ? 0.0 : a.escal * (1e-7 / S * v);
    if (!isfinite(e)) atomicOr(bad, a.form == 2 ? 2 : 1);
    row[p] = e;
  }
}

// ---------------------------------------------------------------------------------
// P rows
// ---------------------------------------------------------------------------------

// check_condition_P_P (compute_row_P_sup.jl:383-394)
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

// face box of Integ_sup_sup_P: intervals from the face centre and extents, the normal
// (smallest extent) length replaced by 1 and always collapsed
__device__ __forceinline__ int face_box(Box& b, const double fc[3], const double ext[3]) {
  for (int d = 0; d < 3; ++d) {
    b.iv[d][0] = fc[d] - ext[d] / 2;
    b.iv[d][1] = fc[d] + ext[d] / 2;
    b.c[d] = fc[d];
    b.len[d] = ext[d];
  }
  const double* e = ext;
  const int nrm = (e[0] <= e[1] && e[0] <= e[2]) ? 0 : ((e[1] <= e[0] && e[1] <= e[2]) ? 1 : 2);
  b.len[nrm] = 1.0;
  return nrm;
}

// Integ_sup_sup_P (compute_row_P_sup.jl:106-381) over two face boxes with normals p1, p2
// (pform 1); pform 4: Song_P_improved_Ivana_strategy (Song_P_improved_Ivana_strategy.jl:
// 1-256), the same tree over the dense RIS surfaces
__device__ double sup_sup_boxes(Box& A, Box& B, int p1, int p2, int pform) {
  const double s1 = A.len[0] * A.len[1] * A.len[2], s2 = B.len[0] * B.len[1] * B.len[2];
  double mxd[3];
  const double min_R = box_gaps(A, B, mxd);
  for (int d = 0; d < 3; ++d) {
    int u, v;
    others(d, u, v);
    A.s[d] = chk_pp(s1, s2, mxd[d], min_R, A.len[d], A.len[u], A.len[v]);
    B.s[d] = chk_pp(s1, s2, mxd[d], min_R, B.len[d], B.len[u], B.len[v]);
  }
  A.s[p1] = 1;
  B.s[p2] = 1;
  A.n = A.s[0] + A.s[1] + A.s[2];
  B.n = B.s[0] + B.s[1] + B.s[2];
  if (A.n + B.n == 2) {  // face - face, the near field
    const double w = A.len[p1] * B.len[p2];
    if (p1 == p2) {
      int u, v;
      others(p1, u, v);
      return w * ss_para(A.iv[u], A.iv[v], A.c[p1], B.iv[u], B.iv[v], B.c[p1]);
    }
    const int a = 3 - p1 - p2;
    return w * ss_ortho(A.iv[a], A.iv[p2], A.c[p1], B.iv[a], B.c[p2], B.iv[p1], pform);
  }
  return integ_boxes(A, B, pform);
}

__device__ double sup_sup(const double f1[3], const double e1[3], const double f2[3],
                          const double e2[3]) {
  Box A, B;
  const int p1 = face_box(A, f1, e1), p2 = face_box(B, f2, e2);
  return sup_sup_boxes(A, B, p1, p2, 1);
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
    const double v = sup_sup(f1, e1, f2, e2);
    const double pref = 1.0 / (4 * pi * eps0 * A1 * d2[0] * d2[1]);
    const double e = a.escal * (pref * v);
    if (!isfinite(e)) atomicOr(bad, 1);
    row[p] = e;
  }
}

// (lattice extents, interleaved axes, caser, caser2) of the six P rows: the QS fill's face
// types (compute_FFT_mutual_coupling_mats.jl:96-125) and those of the Rcc path
// (compute_rows_Rcc_P.jl:47-52), which pass the block indices as face types; the Rcc
// centre distances take the QS face types (compute_rows_Rcc_P.jl:55-60)
struct PDef { int M[3]; int half[3]; int c1, c2, r1, r2; };
static void p_defs(int Nx, int Ny, int Nz, PDef pd[6]) {
  const PDef d[6] = {{{Nx, Ny + 1, Nz}, {0, 0, 0}, 1, 1, 1, 1},
                     {{Nx + 1, Ny, Nz}, {0, 0, 0}, 3, 3, 2, 2},
                     {{Nx, Ny, Nz + 1}, {0, 0, 0}, 5, 5, 3, 3},
                     {{2 * Nx + 1, 2 * Ny + 1, Nz}, {1, 1, 0}, 3, 2, 1, 2},
                     {{Nx, 2 * Ny + 1, 2 * Nz + 1}, {0, 1, 1}, 5, 2, 1, 3},
                     {{2 * Nx + 1, Ny, 2 * Nz + 1}, {1, 0, 1}, 5, 4, 2, 3}};
  for (int r = 0; r < 6; ++r) pd[r] = d[r];
}

// rcc = 0: the QS rows (compute_FFT_mutual_coupling_mats.jl:36-128); rcc = 1: the QS parts
// of the Rcc rows (compute_rows_Rcc_Lp.jl:20-35 over compute_Lp_Voxels_QS,
// compute_rows_Rcc_P.jl:47-52), escaled, Lp self entries zero
static int fill_rows_any(const double origin[3], double sx, double sy, double sz,
                         double escal_Lp, double escal_P, int Nx, int Ny, int Nz,
                         double* const d_rows[9], const int64_t row_len[9], int* d_bad,
                         cudaStream_t st, int rcc) {
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
    a.form = rcc ? 2 : 0;
    k_fill_lp<<<grid, tpb, 0, st>>>(a, d_rows[d], row_len[d], d_bad);
  }
  PDef pd[6];
  p_defs(Nx, Ny, Nz, pd);
  for (int r = 0; r < 6; ++r) {
    if (!d_rows[3 + r] || row_len[3 + r] == 0) continue;
    PRowArgs a;
    a.caser = rcc ? pd[r].r1 : pd[r].c1;
    a.caser2 = rcc ? pd[r].r2 : pd[r].c2;
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

int fill_rows_gpu(const double origin[3], double sx, double sy, double sz, double escal_Lp,
                  double escal_P, int Nx, int Ny, int Nz, double* const d_rows[9],
                  const int64_t row_len[9], int* d_bad, cudaStream_t st) {
  return fill_rows_any(origin, sx, sy, sz, escal_Lp, escal_P, Nx, Ny, Nz, d_rows, row_len, d_bad,
                       st, 0);
}

int fill_rows_rcc_gpu(const double origin[3], double sx, double sy, double sz, double escal_Lp,
                      double escal_P, int Nx, int Ny, int Nz, double* const d_rows[9],
                      const int64_t row_len[9], int* d_bad, cudaStream_t st) {
  return fill_rows_any(origin, sx, sy, sz, escal_Lp, escal_P, Nx, Ny, Nz, d_rows, row_len, d_bad,
                       st, 1);
}

// ---------------------------------------------------------------------------------
// Rcc rows at one frequency: row * exp(-i beta R) (build_row_vox_Rcc.jl:1-11), R the
// distance between the generating cell and each lattice cell: voxel centres for the Lp
// rows (compute_Voxels_Rcc.jl:1-13), face centres of the QS face types for the P rows
// (compute_P_vox_Rcc.jl:1-84). The real and imaginary parts go to separate rows.
// ---------------------------------------------------------------------------------

struct RccRowArgs {
  int lp;            // Lp row (dir) or P row (casers, half)
  int dir;
  int caser, caser2;
  int M[3];
  int half[3];
  double o[3], s[3];
  double beta;
};

__device__ __forceinline__ double norm3(double dx, double dy, double dz) {
  return sqrt(dx * dx + dy * dy + dz * dz);
}

__global__ void k_rcc_phase(RccRowArgs a, const double* __restrict__ qs, double* re, double* im,
                            int64_t N) {
  double c0[3];
  if (a.lp) {
    LpRowArgs l;
    l.dir = a.dir;
    for (int q = 0; q < 3; ++q) { l.o[q] = a.o[q]; l.s[q] = a.s[q]; }
    for (int q = 0; q < 3; ++q) c0[q] = lp_center(l, q, 0);
  } else {
    double e[3], d[2];
    face(a.caser, ctr(a.o[0], a.s[0], 0, a.half[0]), ctr(a.o[1], a.s[1], 0, a.half[1]),
         ctr(a.o[2], a.s[2], 0, a.half[2]), a.s[0], a.s[1], a.s[2], c0, e, d);
  }
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % a.M[0]);
    const int j = (int)((p / a.M[0]) % a.M[1]);
    const int k = (int)(p / ((int64_t)a.M[0] * a.M[1]));
    double c[3];
    if (a.lp) {
      LpRowArgs l;
      l.dir = a.dir;
      for (int q = 0; q < 3; ++q) { l.o[q] = a.o[q]; l.s[q] = a.s[q]; }
      c[0] = lp_center(l, 0, i);
      c[1] = lp_center(l, 1, j);
      c[2] = lp_center(l, 2, k);
    } else {
      double e[3], d[2];
      face(a.caser2, ctr(a.o[0], a.s[0], i, a.half[0]), ctr(a.o[1], a.s[1], j, a.half[1]),
           ctr(a.o[2], a.s[2], k, a.half[2]), a.s[0], a.s[1], a.s[2], c, e, d);
    }
    const double R = norm3(c0[0] - c[0], c0[1] - c[1], c0[2] - c[2]);
    double sn, cs;
    sincos(a.beta * R, &sn, &cs);
    const double v = qs[p];
    re[p] = v * cs;
    im[p] = -(v * sn);
  }
}

// the real and imaginary parts of the nine Rcc rows at propagation constant beta (rad/m)
int rcc_rows_gpu(const double origin[3], double sx, double sy, double sz, int Nx, int Ny, int Nz,
                 double beta, const double* const d_qs[9], double* const d_re[9],
                 double* const d_im[9], const int64_t row_len[9], cudaStream_t st) {
  const int grid = 152 * 8, tpb = 256;
  const int lpM[3][3] = {{Nx - 1, Ny, Nz}, {Nx, Ny - 1, Nz}, {Nx, Ny, Nz - 1}};
  PDef pd[6];
  p_defs(Nx, Ny, Nz, pd);
  for (int r = 0; r < 9; ++r) {
    if (!d_qs[r] || row_len[r] == 0) continue;
    RccRowArgs a;
    a.lp = r < 3;
    a.dir = r < 3 ? r : 0;
    a.caser = r < 3 ? 0 : pd[r - 3].c1;
    a.caser2 = r < 3 ? 0 : pd[r - 3].c2;
    for (int q = 0; q < 3; ++q) {
      a.M[q] = r < 3 ? lpM[r][q] : pd[r - 3].M[q];
      a.half[q] = r < 3 ? 0 : pd[r - 3].half[q];
      a.o[q] = origin[q];
    }
    a.s[0] = sx; a.s[1] = sy; a.s[2] = sz;
    a.beta = beta;
    k_rcc_phase<<<grid, tpb, 0, st>>>(a, d_qs[r], d_re[r], d_im[r], row_len[r]);
  }
  PEEC_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------------
// Dense RIS fill (sharedRis/calcola_Lp.jl, sharedRis/calcola_P.jl): every pair of volumes
// of one current direction (an Lp block) and every pair of surfaces (P), from the bodies'
// vertex coordinates. One thread per pair of a 32 x 32 tile of the upper triangle; each
// tile is written to both triangles of the column-major matrix (padded leading
// dimension), the mirrored half through a shared-memory transpose so that both writes
// are coalesced. FP64 throughout, in the reference's expression order.
// ---------------------------------------------------------------------------------

// calcola_Lp.jl:22-28: the coordinates holding each axis' minimum, then its maximum
__constant__ int c_ris_vol_idx[3][8] = {{0, 6, 12, 18, 3, 9, 15, 21},
                                        {1, 4, 13, 16, 7, 10, 19, 22},
                                        {2, 5, 8, 11, 14, 17, 20, 23}};
// mean_length_rev (Compute_Lp_Self.jl:39-74): the two end faces' vertices per direction
__constant__ int c_ris_ends[3][2][4] = {{{0, 2, 4, 6}, {1, 3, 5, 7}},
                                        {{0, 1, 4, 5}, {2, 3, 6, 7}},
                                        {{0, 1, 2, 3}, {4, 5, 6, 7}}};

// isequal, which Julia's unique uses (0.0 and -0.0 are different values)
__device__ __forceinline__ bool same_value(double a, double b) {
  return a == b && signbit(a) == signbit(b);
}

// calcola_Lp.jl:43-57: per axis the first and the last entry of
// unique(round.(coords[[min; max]], digits=14)), the centre 0.5*(last + first) and the
// length |last - first|
__device__ void ris_vol_box(const double* __restrict__ c24, Box& b) {
  for (int d = 0; d < 3; ++d) {
    double v[8];
    for (int i = 0; i < 8; ++i) v[i] = round14(c24[c_ris_vol_idx[d][i]]);
    double last = v[0];
    for (int i = 1; i < 8; ++i) {
      bool seen = false;
      for (int j = 0; j < i; ++j) seen = seen || same_value(v[i], v[j]);
      if (!seen) last = v[i];
    }
    b.iv[d][0] = v[0];
    b.iv[d][1] = last;
    b.c[d] = 0.5 * (last + v[0]);
    b.len[d] = fabs(last - v[0]);
  }
}

// mean_length_rev (Compute_Lp_Self.jl:39-74): the distance between the centroids of the
// brick's two end faces along direction dir (1, 2, 3)
__device__ double mean_length_rev(const double* __restrict__ c24, int dir) {
  double d2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < 4; ++i) {
      a = a + c24[3 * c_ris_ends[dir - 1][0][i] + k];
      b = b + c24[3 * c_ris_ends[dir - 1][1][i] + k];
    }
    const double e = 0.25 * a - 0.25 * b;
    d2 += e * e;
  }
  return sqrt(d2);
}

// Compute_Lp_Self (Compute_Lp_Self.jl:1-37): the closed-form self inductance of a bar of
// length l, width W, thickness T; 0 when 1/(l W T) is not finite
__device__ double lp_self(double l, double W, double T) {
  if (!isfinite(1.0 / (l * W * T))) return 0.0;
  const double w = W / l, t = T / l;
  const double r = sqrt(w * w + t * t), aw = sqrt(w * w + 1), at = sqrt(t * t + 1);
  const double ar = sqrt(w * w + t * t + 1);
  const double mu0 = 4 * CUDART_PI * 1e-7;
  const double g1 = 1.0 / 4 * (1 / w * asinh(w / at) + 1 / t * asinh(t / aw) + asinh(1 / r));
  const double g2 =
      1.0 / 24 *
      (t * t / w * asinh(w / (t * at * (r + ar))) + w * w / t * asinh(t / (w * aw * (r + ar))) +
       t * t / (w * w) * asinh(w * w / (t * r * (at + ar))) +
       w * w / (t * t) * asinh(t * t / (w * r * (aw + ar))) +
       1 / (w * (t * t)) * asinh(w * (t * t) / (at * (aw + ar))) +
       1 / (t * (w * w)) * asinh(t * (w * w) / (aw * (at + ar))));
  const double g3 =
      1.0 / 6 * (1 / (w * t) * atan(w * t / ar) + t / w * atan(w / (t * ar)) + w / t * atan(t / (w * ar)));
  const double g4 = 1.0 / 60 *
                    ((ar + r + t + at) * (t * t) / ((ar + r) * (r + t) * (t + at) * (at + ar)) +
                     (ar + r + w + aw) * (w * w) / ((ar + r) * (r + w) * (w + aw) * (aw + ar)) +
                     (ar + aw + 1 + at) / ((ar + aw) * (aw + 1) * (1 + at) * (at + ar)));
  const double g5 = 1.0 / 20 * (1 / (r + ar) + 1 / (aw + ar) + 1 / (at + ar));
  return 2 * mu0 * l / CUDART_PI * (g1 + g2 - g3 - g4 - g5);
}

// per volume: its box and its self inductance (calcola_Lp.jl:43-77; the current
// direction from the volume's index: x for the first mx volumes, then y, then z)
__global__ void k_ris_vol_prep(const double* __restrict__ coords, int64_t m, int64_t mx,
                               int64_t my, Box* __restrict__ out, double* __restrict__ self) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double* c = coords + 24 * i;
    Box b;
    ris_vol_box(c, b);
    b.s[0] = b.s[1] = b.s[2] = 0;
    b.n = 0;
    out[i] = b;
    const int dir = i < mx ? 1 : (i < mx + my ? 2 : 3);
    const double m1 = fabs(mean_length_rev(c, 1)), m2 = fabs(mean_length_rev(c, 2)),
                 m3 = fabs(mean_length_rev(c, 3));
    double l, W, T;
    if (dir == 1) { l = m1; W = m3; T = m2; }
    else if (dir == 2) { T = m1; W = m3; l = m2; }
    else { W = m1; l = m3; T = m2; }
    self[i] = lp_self(l, W, T);
  }
}

// per surface (process_surfaces!, calcola_P.jl:94-160): the box from vertices 1 and 4,
// rounded, the normal (the smallest extent) given length 1
__global__ void k_ris_surf_prep(const double* __restrict__ ends, int64_t ns, Box* __restrict__ out,
                                int* __restrict__ nrm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ns;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double* e = ends + 12 * i;
    Box b;
    for (int d = 0; d < 3; ++d) {
      const double p = e[d], q = e[9 + d];
      b.iv[d][0] = round14(fmin(p, q));
      b.iv[d][1] = round14(fmax(p, q));
      b.c[d] = 0.5 * (b.iv[d][1] + b.iv[d][0]);
      b.len[d] = fabs(b.iv[d][1] - b.iv[d][0]);
    }
    const double* l = b.len;
    const int k = (l[0] <= l[1] && l[0] <= l[2]) ? 0 : ((l[1] <= l[0] && l[1] <= l[2]) ? 1 : 2);
    b.len[k] = 1.0;
    b.s[0] = b.s[1] = b.s[2] = 0;
    b.n = 0;
    out[i] = b;
    nrm[i] = k;
  }
}

// One block of the dense fill: its bodies (with their normals for P), cross-sections or
// areas, self terms (Lp), size and output matrix.
struct RisBlock {
  const Box* bodies;
  const int* nrm;
  const double* S;
  const double* self;
  int64_t dim;
  double* M;
  int64_t ld;
};
struct RisBlocks {
  RisBlock b[3];
};

// KIND 0: an Lp block (Song_improved_Ivana_strategy2 off the diagonal, the self term
// on it, 1e-7 / (S_m S_n) * integral * esc; calculate_Lp_matrix, calcola_Lp.jl:254-306);
// KIND 1: P (Song_P_improved_Ivana_strategy on and off the diagonal,
// integral / (4 pi eps0 S_m S_n) * esc; calculate_P_matrix, calcola_P.jl:162-222).
// Grid (tiles, tiles, blocks): CTA (x, y, z) takes the T x T tile of rows Ty.. and columns
// Tx.. of block z, x >= y; 256 threads, T*T/256 pairs each. The three Lp blocks share one
// launch, and small blocks take T = 16, so that the GPU fills with CTAs.
template <int KIND, int T>
__global__ void __launch_bounds__(256) k_ris_pairs(RisBlocks blocks, double esc, int* bad) {
  constexpr int ROWS = 256 / T;
  __shared__ Box rb[T], cb[T];
  __shared__ int rn[T], cn[T];
  __shared__ double tile[T][T + 1];
  const RisBlock& blk = blocks.b[blockIdx.z];
  const int64_t dim = blk.dim, ld = blk.ld;
  const int64_t ti = blockIdx.y, tj = blockIdx.x;
  if (ti > tj || tj * T >= dim) return;
  const int tx = threadIdx.x % T, ty = threadIdx.x / T;
  const int64_t m0 = ti * T, n0 = tj * T;
  if (ty == 0 && m0 + tx < dim) {
    rb[tx] = blk.bodies[m0 + tx];
    rn[tx] = KIND ? blk.nrm[m0 + tx] : 0;
  } else if (ty == 1 && n0 + tx < dim) {
    cb[tx] = blk.bodies[n0 + tx];
    cn[tx] = KIND ? blk.nrm[n0 + tx] : 0;
  }
  __syncthreads();
  const double pi = CUDART_PI;
  const double eps0 = 8.854187816997944e-12;
  const double* S = blk.S;
  double* M = blk.M;
  const int64_t m = m0 + tx;
  for (int k = 0; k < T / ROWS; ++k) {
    const int nl = ty + ROWS * k;
    const int64_t n = n0 + nl;
    double e = 0.0;
    if (m < dim && n < dim && (KIND ? m <= n : m < n)) {
      Box A = rb[tx], B = cb[nl];
      double v;
      if (KIND == 0) {
        lp_flags(A, B);
        v = (A.n + B.n == 0) ? vol_vol(A.iv[0], A.iv[1], A.iv[2], B.iv[0], B.iv[1], B.iv[2])
                             : integ_boxes(A, B, 3);
        e = 1e-7 / (S[m] * S[n]) * v * esc;
      } else {
        v = sup_sup_boxes(A, B, rn[tx], cn[nl], 4);
        e = 1.0 / (4 * pi * eps0 * S[m] * S[n]) * v * esc;
      }
      if (!isfinite(e)) atomicAdd(bad, 1);
      M[m + n * ld] = e;
    }
    tile[nl][tx] = e;
  }
  __syncthreads();
  for (int k = 0; k < T / ROWS; ++k) {  // the mirrored entries (n, m), m < n
    const int ml = ty + ROWS * k;
    const int64_t mm = m0 + ml, nn = n0 + tx;
    if (mm < dim && nn < dim && mm < nn) M[nn + mm * ld] = tile[tx][ml];
  }
  if (KIND == 0 && ti == tj && ty == 0 && m < dim) {
    const double e = blk.self[m] * esc;
    if (!isfinite(e)) atomicAdd(bad, 1);
    M[m + m * ld] = e;
  }
}

// centre distances (calculate_Rx / _Ry / _Rz, calcola_Lp.jl:99-252; calculate_R_cc!,
// calcola_P.jl:49-92): R[m, n] = |c_m - c_n|, column-major, leading dimension ld
__global__ void k_ris_dist(const double* __restrict__ ctr, int64_t dim, double* __restrict__ R,
                           int64_t ld) {
  for (int64_t n = blockIdx.y; n < dim; n += gridDim.y) {
    const double x = ctr[3 * n], y = ctr[3 * n + 1], z = ctr[3 * n + 2];
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < dim;
         m += (int64_t)gridDim.x * blockDim.x) {
      const double dx = ctr[3 * m] - x, dy = ctr[3 * m + 1] - y, dz = ctr[3 * m + 2] - z;
      R[m + n * ld] = sqrt(dx * dx + dy * dy + dz * dz);
    }
  }
}

__global__ void k_inv_diag(const double* __restrict__ M, int64_t ld, int64_t n,
                           double* __restrict__ inv) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    inv[i] = 1.0 / M[i + i * ld];
}

size_t ris_box_bytes() { return sizeof(Box); }

// The bodies' boxes (and the volumes' self terms) into the scratch: boxes (count Box),
// self (count doubles, volumes) or nrm (count ints, surfaces)
int ris_prep_gpu(int surfaces, const double* d_geom, int64_t count, int64_t mx, int64_t my,
                 void* boxes, double* self, int* nrm, cudaStream_t st) {
  if (count <= 0) return 0;
  const int tpb = 128;
  const int blocks = (int)std::min<int64_t>((count + tpb - 1) / tpb, 152 * 16);
  if (surfaces)
    k_ris_surf_prep<<<blocks, tpb, 0, st>>>(d_geom, count, (Box*)boxes, nrm);
  else
    k_ris_vol_prep<<<blocks, tpb, 0, st>>>(d_geom, count, mx, my, (Box*)boxes, self);
  PEEC_CUDA_TRY(cudaGetLastError());
  return 0;
}

// the dense blocks of one fill: kind 0, up to three Lp blocks in one launch (boxes, self
// terms and S of their volumes); kind 1, P. M zeroed by the caller (padding rows stay zero).
template <int KIND, int T>
static void launch_pairs(const RisBlocks& rb, int nb, int64_t nt, double esc, int* d_bad,
                         cudaStream_t st) {
  const dim3 grid((unsigned)nt, (unsigned)nt, (unsigned)nb);
  k_ris_pairs<KIND, T><<<grid, 256, 0, st>>>(rb, esc, d_bad);
}

int ris_pairs_gpu(int kind, int nb, const void* const* boxes, const int* nrm,
                  const double* const* S, const double* const* self, const int64_t* dim,
                  double esc, double* const* M, const int64_t* ld, int* d_bad, cudaStream_t st) {
  RisBlocks rb;
  int64_t maxdim = 0, tiles32 = 0;
  for (int b = 0; b < 3; ++b) {
    const bool on = b < nb;
    rb.b[b] = RisBlock{on ? (const Box*)boxes[b] : nullptr, kind ? nrm : nullptr,
                       on ? S[b] : nullptr, on ? (self ? self[b] : nullptr) : nullptr,
                       on ? dim[b] : 0, on ? M[b] : nullptr, on ? ld[b] : 1};
    if (on) {
      maxdim = std::max(maxdim, dim[b]);
      const int64_t t = (dim[b] + 31) / 32;
      tiles32 += t * (t + 1) / 2;
    }
  }
  if (maxdim <= 0) return 0;
  // 32 x 32 tiles once they give every SM a few CTAs, else 16 x 16
  const bool big = tiles32 >= 152 * 4;
  const int T = big ? 32 : 16;
  const int64_t nt = (maxdim + T - 1) / T;
  if (nt > 65535) return PEEC_ERR_UNSUPPORTED_INTERNAL;
  if (kind == 0) {
    if (big) launch_pairs<0, 32>(rb, nb, nt, esc, d_bad, st);
    else launch_pairs<0, 16>(rb, nb, nt, esc, d_bad, st);
  } else {
    if (big) launch_pairs<1, 32>(rb, nb, nt, esc, d_bad, st);
    else launch_pairs<1, 16>(rb, nb, nt, esc, d_bad, st);
  }
  PEEC_CUDA_TRY(cudaGetLastError());
  return 0;
}

int ris_dist_gpu(const double* d_ctr, int64_t dim, double* R, int64_t ld, cudaStream_t st) {
  if (dim <= 0) return 0;
  const int tpb = 256;
  const dim3 grid((unsigned)std::min<int64_t>((dim + tpb - 1) / tpb, 64),
                  (unsigned)std::min<int64_t>(dim, 65535));
  k_ris_dist<<<grid, tpb, 0, st>>>(d_ctr, dim, R, ld);
  PEEC_CUDA_TRY(cudaGetLastError());
  return 0;
}

int inv_diag_gpu(const double* M, int64_t ld, int64_t n, double* inv, cudaStream_t st) {
  if (n <= 0) return 0;
  const int tpb = 256;
  k_inv_diag<<<(unsigned)std::min<int64_t>((n + tpb - 1) / tpb, 1024), tpb, 0, st>>>(M, ld, n, inv);
  PEEC_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace peec
