/*
 * ORACLE -- test infrastructure only. CPU restatement of the reference's voxel
 * Lp / P generating-row fill, used by tests/ and bench.py's cpu_baseline leg as
 * the checker; never linked into the product.
 *
 * Built twice by oracle/build.py: REAL=double (suffix _d) and REAL=long double
 * (suffix _ld); the long double build is the high-precision evaluation of the
 * same formulas the fill parity tests measure both CPU and GPU rows against.
 *
 * Follows:
 *   src/lib/solverFFT/compute_Lp_Voxels.jl:1-63    row driver (round_ud_fft :807)
 *   src/lib/solverFFT/compute_Lp_Voxels.jl:65-306  Integ_vol_vol_fft dispatch
 *   src/lib/solverFFT/compute_Lp_Voxels.jl:437-447 check_condition_fft
 *   src/lib/solverFFT/compute_Lp_Voxels.jl:766-805 integ_vol_vol_fft
 *   src/lib/solverFFT/compute_row_P_sup.jl:1-104   row driver (caser/caser2)
 *   src/lib/solverFFT/compute_row_P_sup.jl:106-381 Integ_sup_sup_P dispatch
 *   src/lib/solverFFT/compute_row_P_sup.jl:383-394 check_condition_P_P
 *   src/lib/solverFFT/compute_row_P_sup.jl:557-590 integ_surf_surf_ortho_P
 *   src/lib/solverFFT/compute_Lp_Voxels_QS.jl:695-730 integ_surf_surf_para
 * Only the near-field branches (no suppression: volume-volume for Lp,
 * surface-surface for P) are restated; an entry whose suppression test fires is
 * returned as NaN and counted, so a caller can never take a far-field entry from
 * here silently. On uniform voxels the suppression tests need centre distances
 * above ~200 voxel edges, beyond every grid the tests and benchmarks use.
 *
 * Besides the value each entry also returns the sum of |terms| of its closed
 * form (times the same prefactor): the cancellation-aware scale for error bounds.
 */
#include <math.h>
#include <stdint.h>

#ifndef REAL
#define REAL double
#endif
#ifndef SFX
#define SFX _d
#endif
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

#ifdef LONGD
#define SQRT sqrtl
#define LOG logl
#define ATAN2 atan2l
#define FABS fabsl
#define RINT nearbyintl
#define ISFIN isfinite
#else
#define SQRT sqrt
#define LOG log
#define ATAN2 atan2
#define FABS fabs
#define RINT nearbyint
#define ISFIN isfinite
#endif

/* real(log(complex(v))) for v >= 0; -inf at 0 (the callers zero a non-finite term) */
static REAL lg(REAL v) { return v > 0 ? LOG(v) : (v == 0 ? -INFINITY : LOG(FABS(v))); }
static REAL fin(REAL t) { return ISFIN(t) ? t : 0; }
static REAL sgnp(int s) { return (s & 1) ? -1 : 1; }

/* round_ud_fft(v, 14): round(v*10^14)/10^14, ties to even (compute_Lp_Voxels.jl:807) */
static REAL round14(REAL v) { return RINT(v * (REAL)1e14) / (REAL)1e14; }

static int check_fft(REAL e1, REAL e2, REAL e3, REAL V1, REAL V2, REAL max_d, REAL min_R,
                     REAL size_dim, REAL o1, REAL o2) {
  REAL max_oth = o1 > o2 ? o1 : o2;
  REAL a = V1 * V2 * max_d / ((min_R + (REAL)1e-15) * (min_R + (REAL)1e-15) * (min_R + (REAL)1e-15));
  REAL f = size_dim / (min_R + (REAL)1e-15);
  REAL b = size_dim / max_oth;
  return ((b <= e3 || f < e1) && a < e2) ? 1 : 0;
}

static REAL maxabs4(REAL a, REAL b, REAL c, REAL d) {
  REAL m = FABS(a);
  if (FABS(b) > m) m = FABS(b);
  if (FABS(c) > m) m = FABS(c);
  if (FABS(d) > m) m = FABS(d);
  return m;
}
static REAL minabs4(REAL a, REAL b, REAL c, REAL d) {
  REAL m = FABS(a);
  if (FABS(b) < m) m = FABS(b);
  if (FABS(c) < m) m = FABS(c);
  if (FABS(d) < m) m = FABS(d);
  return m;
}

/* integ_vol_vol_fft: 64-term closed form; *abssum gets sum |term| */
static REAL vol_vol(const REAL* x1v, const REAL* y1v, const REAL* z1v, const REAL* x2v,
                    const REAL* y2v, const REAL* z2v, REAL* abssum) {
  REAL sol = 0, acc = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3)
        for (int c4 = 0; c4 < 2; ++c4)
          for (int c5 = 0; c5 < 2; ++c5)
            for (int c6 = 0; c6 < 2; ++c6) {
              REAL X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2v[c5], Z = z1v[c3] - z2v[c6];
              REAL X2 = X * X, Y2 = Y * Y, Z2 = Z * Z;
              REAL R = SQRT(X2 + Y2 + Z2);
              REAL t1 = (X2 * X2 + Y2 * Y2 + Z2 * Z2 - 3 * X2 * Y2 - 3 * Y2 * Z2 - 3 * X2 * Z2) * R / 60;
              REAL t2 = fin((Y2 * Z2 / 4 - Y2 * Y2 / 24 - Z2 * Z2 / 24) * X * lg(X + R));
              REAL t3 = fin((Y2 * X2 / 4 - Y2 * Y2 / 24 - X2 * X2 / 24) * Z * lg(Z + R));
              REAL t4 = fin((Z2 * X2 / 4 - Z2 * Z2 / 24 - X2 * X2 / 24) * Y * lg(Y + R));
              REAL t5 = -FABS(X) * X2 * Y * Z / 6 * ATAN2(Y * Z, FABS(X) * R);
              REAL t6 = -X * FABS(Y) * Y2 * Z / 6 * ATAN2(X * Z, FABS(Y) * R);
              REAL t7 = -X * Y * FABS(Z) * Z2 / 6 * ATAN2(X * Y, FABS(Z) * R);
              REAL s = t1 + t2 + t3 + t4 + t5 + t6 + t7;
              /* (-1)^(c1+..+c6+1) with 1-based c's = (-1)^(sum0 + 1) */
              sol += sgnp(c1 + c2 + c3 + c4 + c5 + c6 + 1) * s;
              acc += FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4) + FABS(t5) + FABS(t6) + FABS(t7);
            }
  *abssum = acc;
  return sol;
}

/* Integ_vol_vol_fft suppression tests; returns the number of suppressed dims */
static int lp_supp(const REAL* x1v, const REAL* y1v, const REAL* z1v, const REAL* x2v,
                   const REAL* y2v, const REAL* z2v) {
  const REAL e1 = 5e-3, e2 = 1e-3, e3 = 1e-3, e4 = 3e-1;
  REAL a1 = FABS(x1v[1] - x1v[0]), b1 = FABS(y1v[1] - y1v[0]), c1 = FABS(z1v[1] - z1v[0]);
  REAL a2 = FABS(x2v[1] - x2v[0]), b2 = FABS(y2v[1] - y2v[0]), c2 = FABS(z2v[1] - z2v[0]);
  REAL V1 = a1 * b1 * c1, V2 = a2 * b2 * c2;
  REAL ax[4] = {x1v[0] - x2v[0], x1v[0] - x2v[1], x1v[1] - x2v[0], x1v[1] - x2v[1]};
  REAL ay[4] = {y1v[0] - y2v[0], y1v[0] - y2v[1], y1v[1] - y2v[0], y1v[1] - y2v[1]};
  REAL az[4] = {z1v[0] - z2v[0], z1v[0] - z2v[1], z1v[1] - z2v[0], z1v[1] - z2v[1]};
  REAL mx = minabs4(ax[0], ax[1], ax[2], ax[3]), my = minabs4(ay[0], ay[1], ay[2], ay[3]),
       mz = minabs4(az[0], az[1], az[2], az[3]);
  REAL min_R = SQRT(mx * mx + my * my + mz * mz);
  REAL dx = maxabs4(ax[0], ax[1], ax[2], ax[3]), dy = maxabs4(ay[0], ay[1], ay[2], ay[3]),
       dz = maxabs4(az[0], az[1], az[2], az[3]);
  int s = 0;
  for (int side = 0; side < 2; ++side) {
    REAL a = side ? a2 : a1, b = side ? b2 : b1, c = side ? c2 : c1;
    int sx = 0, sy = 0, sz = 0;
    if (a <= b && a <= c) {
      sx = check_fft(e1, e2, e3, V1, V2, dx, min_R, a, b, c);
      if (sx && (b > c ? b : c) / (min_R + (REAL)1e-15) < e4) {
        sy = check_fft(e1, e2, e3, V1, V2, dy, min_R, b, a, c);
        sz = check_fft(e1, e2, e3, V1, V2, dz, min_R, c, a, b);
      }
    } else if (b <= a && b <= c) {
      sy = check_fft(e1, e2, e3, V1, V2, dy, min_R, b, a, c);
      if (sy && (a > c ? a : c) / (min_R + (REAL)1e-15) < e4) {
        sx = check_fft(e1, e2, e3, V1, V2, dx, min_R, a, b, c);
        sz = check_fft(e1, e2, e3, V1, V2, dz, min_R, c, a, b);
      }
    } else {
      sz = check_fft(e1, e2, e3, V1, V2, dz, min_R, c, a, b);
      if (sz && (a > b ? a : b) / (min_R + (REAL)1e-15) < e4) {
        sx = check_fft(e1, e2, e3, V1, V2, dx, min_R, a, b, c);
        sy = check_fft(e1, e2, e3, V1, V2, dy, min_R, b, a, c);
      }
    }
    s += sx + sy + sz;
  }
  return s;
}

/* One Lp generating row: source centre src, targets centers[N][3] (row-major),
 * current direction dc = 1,2,3. out[k] = 1e-7/S * integral (compute_Lp_Voxels.jl:40-60),
 * scale[k] = the same prefactor times sum|terms|. Returns the count of entries
 * that needed a far-field branch (set to NaN). */
int64_t FN(oracle_lp_row)(int dc, const double* src, const double* centers, int64_t N,
                          double sx_, double sy_, double sz_, double* out, double* scale) {
  REAL sx = sx_, sy = sy_, sz = sz_;
  REAL S = sy * sz * sy * sz;
  if (dc == 2) S = sx * sz * sx * sz;
  else if (dc == 3) S = sx * sy * sx * sy;
  REAL c1x = src[0], c1y = src[1], c1z = src[2];
  REAL x1v[2] = {round14(c1x - sx / 2), round14(c1x + sx / 2)};
  REAL y1v[2] = {round14(c1y - sy / 2), round14(c1y + sy / 2)};
  REAL z1v[2] = {round14(c1z - sz / 2), round14(c1z + sz / 2)};
  int64_t bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int64_t k = 0; k < N; ++k) {
    REAL cx = centers[3 * k], cy = centers[3 * k + 1], cz = centers[3 * k + 2];
    REAL x2v[2] = {round14(cx - sx / 2), round14(cx + sx / 2)};
    REAL y2v[2] = {round14(cy - sy / 2), round14(cy + sy / 2)};
    REAL z2v[2] = {round14(cz - sz / 2), round14(cz + sz / 2)};
    if (lp_supp(x1v, y1v, z1v, x2v, y2v, z2v) != 0) {
      out[k] = NAN;
      if (scale) scale[k] = NAN;
      bad += 1;
      continue;
    }
    REAL acc;
    REAL v = vol_vol(x1v, y1v, z1v, x2v, y2v, z2v, &acc);
    out[k] = (double)((REAL)1e-7 / S * v);
    if (scale) scale[k] = (double)((REAL)1e-7 / S * acc);
  }
  return bad;
}

/* integ_surf_surf_para (compute_Lp_Voxels_QS.jl:695-730) */
static REAL ss_para(const REAL* x1v, const REAL* y1v, REAL z1, const REAL* x2v, const REAL* y2v,
                    REAL z2, REAL* abssum) {
  REAL sol = 0, acc = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3)
        for (int c4 = 0; c4 < 2; ++c4) {
          REAL X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2v[c3], Z = z1 - z2;
          REAL R = SQRT(X * X + Y * Y + Z * Z);
          REAL t1 = -(REAL)1 / 6 * (X * X + Y * Y - 2 * Z * Z) * R;
          REAL t2 = -X * Y * FABS(Z) * ATAN2(X * Y, FABS(Z) * R);
          REAL t3 = fin((REAL)0.5 * (X * X - Z * Z) * Y * lg(Y + R));
          REAL t4 = fin((REAL)0.5 * (Y * Y - Z * Z) * X * lg(X + R));
          sol += sgnp(c1 + c2 + c3 + c4) * (t1 + t2 + t3 + t4);
          acc += FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4);
        }
  *abssum = acc;
  return sol;
}

/* integ_surf_surf_ortho_P (compute_row_P_sup.jl:557-590) */
static REAL ss_ortho(const REAL* x1v, const REAL* y1v, REAL z1, const REAL* x2v, REAL y2,
                     const REAL* z2v, REAL* abssum) {
  REAL sol = 0, acc = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3)
        for (int c4 = 0; c4 < 2; ++c4) {
          REAL X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2, Z = z1 - z2v[c3];
          REAL R = SQRT(X * X + Y * Y + Z * Z);
          REAL t1 = -(REAL)1 / 3 * Y * Z * R;
          REAL t2 = -(REAL)0.5 * X * FABS(Z) * Z * ATAN2(X * Y, FABS(Z) * R);
          REAL t3 = -(REAL)0.5 * X * FABS(Y) * Y * ATAN2(X * Z, FABS(Y) * R);
          REAL t4 = -(REAL)1 / 6 * FABS(X) * X * X * ATAN2(Y * Z, FABS(X) * R);
          REAL t5 = fin(X * Y * Z * lg(X + R));
          REAL t6 = fin(((REAL)0.5 * X * X - (REAL)1 / 6 * Z * Z) * Z * lg(Y + R));
          REAL t7 = fin(((REAL)0.5 * X * X - (REAL)1 / 6 * Y * Y) * Y * lg(Z + R));
          sol += sgnp(c1 + c2 + c3 + c4) * (t1 + t2 + t3 + t4 + t5 + t6 + t7);
          acc += FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4) + FABS(t5) + FABS(t6) + FABS(t7);
        }
  *abssum = acc;
  return sol;
}

static int check_pp(REAL e1, REAL e2, REAL e3, REAL e4, REAL S1, REAL S2, REAL max_d, REAL min_R,
                    REAL size_dim, REAL o1, REAL o2) {
  REAL max_oth = o1 * o2;
  REAL condS = (max_oth > size_dim ? max_oth : size_dim) / (min_R + (REAL)1e-15);
  REAL mr = min_R + (REAL)1e-15;
  REAL a = S1 * S2 * max_d / (mr * mr * mr);
  REAL f = size_dim / mr;
  REAL b = size_dim / max_oth;
  return (condS < e4 && (b <= e3 || f < e1) && a < e2) ? 1 : 0;
}

/* Integ_sup_sup_P restricted to the surface-surface branch; returns NaN (and
 * *unsup=1) when a suppression test fires. */
static REAL sup_sup(REAL xc1, REAL yc1, REAL zc1, REAL xc2, REAL yc2, REAL zc2, REAL a1, REAL b1,
                    REAL c1, REAL a2, REAL b2, REAL c2, REAL* abssum, int* unsup) {
  const REAL e1 = 5e-3, e2 = 1e-3, e3 = 1e-3, e4 = 3e-1;
  REAL x1v[2] = {xc1 - a1 / 2, xc1 + a1 / 2}, y1v[2] = {yc1 - b1 / 2, yc1 + b1 / 2},
       z1v[2] = {zc1 - c1 / 2, zc1 + c1 / 2};
  REAL x2v[2] = {xc2 - a2 / 2, xc2 + a2 / 2}, y2v[2] = {yc2 - b2 / 2, yc2 + b2 / 2},
       z2v[2] = {zc2 - c2 / 2, zc2 + c2 / 2};
  int p1 = 2, p2 = 2; /* normal axis: 0 yz-plane, 1 xz-plane, 2 xy-plane */
  if (a1 <= b1 && a1 <= c1) { p1 = 0; a1 = 1; }
  else if (b1 <= a1 && b1 <= c1) { p1 = 1; b1 = 1; }
  else { c1 = 1; }
  if (a2 <= b2 && a2 <= c2) { p2 = 0; a2 = 1; }
  else if (b2 <= a2 && b2 <= c2) { p2 = 1; b2 = 1; }
  else { c2 = 1; }
  REAL s1 = a1 * b1 * c1, s2 = a2 * b2 * c2;
  REAL ax[4] = {x1v[0] - x2v[0], x1v[0] - x2v[1], x1v[1] - x2v[0], x1v[1] - x2v[1]};
  REAL ay[4] = {y1v[0] - y2v[0], y1v[0] - y2v[1], y1v[1] - y2v[0], y1v[1] - y2v[1]};
  REAL az[4] = {z1v[0] - z2v[0], z1v[0] - z2v[1], z1v[1] - z2v[0], z1v[1] - z2v[1]};
  REAL mx = minabs4(ax[0], ax[1], ax[2], ax[3]), my = minabs4(ay[0], ay[1], ay[2], ay[3]),
       mz = minabs4(az[0], az[1], az[2], az[3]);
  REAL min_R = SQRT(mx * mx + my * my + mz * mz);
  REAL dx = maxabs4(ax[0], ax[1], ax[2], ax[3]), dy = maxabs4(ay[0], ay[1], ay[2], ay[3]),
       dz = maxabs4(az[0], az[1], az[2], az[3]);
  int sx1 = check_pp(e1, e2, e3, e4, s1, s2, dx, min_R, a1, b1, c1);
  int sx2 = check_pp(e1, e2, e3, e4, s1, s2, dx, min_R, a2, b2, c2);
  int sy1 = check_pp(e1, e2, e3, e4, s1, s2, dy, min_R, b1, a1, c1);
  int sy2 = check_pp(e1, e2, e3, e4, s1, s2, dy, min_R, b2, a2, c2);
  int sz1 = check_pp(e1, e2, e3, e4, s1, s2, dz, min_R, c1, a1, b1);
  int sz2 = check_pp(e1, e2, e3, e4, s1, s2, dz, min_R, c2, a2, b2);
  if (p1 == 0) sx1 = 1; else if (p1 == 1) sy1 = 1; else sz1 = 1;
  if (p2 == 0) sx2 = 1; else if (p2 == 1) sy2 = 1; else sz2 = 1;
  if (sx1 + sy1 + sz1 + sx2 + sy2 + sz2 != 2) {
    *unsup = 1;
    *abssum = NAN;
    return NAN;
  }
  REAL X1[2], Y1[2], X2[2], Z2[2];
  if (p1 == 0) {
    if (p2 == 0) return a1 * a2 * ss_para(y1v, z1v, xc1, y2v, z2v, xc2, abssum);
    if (p2 == 1) return a1 * b2 * ss_ortho(z1v, y1v, xc1, z2v, yc2, x2v, abssum);
    return a1 * c2 * ss_ortho(y1v, z1v, xc1, y2v, zc2, x2v, abssum);
  }
  if (p1 == 1) {
    if (p2 == 0) return b1 * a2 * ss_ortho(z1v, x1v, yc1, z2v, xc2, y2v, abssum);
    if (p2 == 1) return b1 * b2 * ss_para(x1v, z1v, yc1, x2v, z2v, yc2, abssum);
    return b1 * c2 * ss_ortho(x1v, z1v, yc1, x2v, zc2, y2v, abssum);
  }
  (void)X1; (void)Y1; (void)X2; (void)Z2;
  if (p2 == 0) return c1 * a2 * ss_ortho(y1v, x1v, zc1, y2v, xc2, z2v, abssum);
  if (p2 == 1) return c1 * b2 * ss_ortho(x1v, y1v, zc1, x2v, yc2, z2v, abssum);
  return c1 * c2 * ss_para(x1v, y1v, zc1, x2v, y2v, zc2, abssum);
}

/* face centre and extents of face type caser (1..6) of a voxel centred at c
 * (compute_row_P_sup.jl:3-51 and the caser2 branches :54-102) */
static void face(int caser, REAL cx, REAL cy, REAL cz, REAL sx, REAL sy, REAL sz, REAL* fc,
                 REAL* ext, REAL* d) {
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

/* One P generating row (compute_row_P_sup.jl:1-104): source centre src with face
 * caser, targets centers[N][3] with face caser2. out is escaled by escal_P. */
int64_t FN(oracle_p_row)(int caser, int caser2, const double* src, const double* centers,
                         int64_t N, double sx_, double sy_, double sz_, double escal_P,
                         double* out, double* scale) {
  const REAL eps0 = 8.854187816997944e-12L;
  const REAL pi = 3.14159265358979323846264338327950288L;
  REAL sx = sx_, sy = sy_, sz = sz_;
  REAL f1[3], e1[3], d1[2];
  face(caser, src[0], src[1], src[2], sx, sy, sz, f1, e1, d1);
  REAL A1 = d1[0] * d1[1];
  int64_t bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int64_t k = 0; k < N; ++k) {
    REAL f2[3], e2[3], d2[2];
    face(caser2, centers[3 * k], centers[3 * k + 1], centers[3 * k + 2], sx, sy, sz, f2, e2, d2);
    REAL acc;
    int unsup = 0;
    REAL v = sup_sup(f1[0], f1[1], f1[2], f2[0], f2[1], f2[2], e1[0], e1[1], e1[2], e2[0], e2[1],
                     e2[2], &acc, &unsup);
    /* 1/(4*pi*eps0*A1*d*d) evaluated left to right as the reference writes it */
    REAL pref = (REAL)1 / ((REAL)4 * pi * eps0 * A1 * d2[0] * d2[1]);
    if (unsup) {
      out[k] = NAN;
      if (scale) scale[k] = NAN;
      bad += 1;
      continue;
    }
    out[k] = (double)((REAL)escal_P * (pref * v));
    if (scale) scale[k] = (double)((REAL)escal_P * (pref * acc));
  }
  return bad;
}
