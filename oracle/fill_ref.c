/*
 * ORACLE -- test infrastructure only. CPU restatement of the reference's voxel
 * Lp / P generating-row fill, used by tests/ and bench.py's cpu_baseline leg as
 * the checker; never linked into the product.
 *
 * Parity unpinned: the reference (Julia) cannot run here and ships no outputs for
 * this path; the rows are held to closed forms (coincident-cell self terms, the
 * far-field point limit) by tests/test_oracle_known_answers.py.
 *
 * Built twice by oracle/build.py: REAL=double (suffix _d) and REAL=long double
 * (suffix _ld); the long double build is the high-precision evaluation of the
 * same formulas the fill parity tests measure both CPU and GPU rows against.
 *
 * Follows:
 *   src/lib/solverFFT/compute_Lp_Voxels.jl:1-63    row driver (round_ud_fft :807)
 *   src/lib/solverFFT/compute_Lp_Voxels.jl:65-435  Integ_vol_vol_fft dispatch
 *   src/lib/solverFFT/compute_Lp_Voxels.jl:437-447 check_condition_fft
 *   src/lib/solverFFT/compute_Lp_Voxels.jl:449-805 primitives (integ_*_fft)
 *   src/lib/solverFFT/compute_row_P_sup.jl:1-104   row driver (caser/caser2)
 *   src/lib/solverFFT/compute_row_P_sup.jl:106-381 Integ_sup_sup_P dispatch
 *   src/lib/solverFFT/compute_row_P_sup.jl:383-394 check_condition_P_P
 *   src/lib/solverFFT/compute_row_P_sup.jl:396-590 primitives (integ_*_P)
 *   src/lib/solverFFT/compute_Lp_Voxels_QS.jl:695-730 integ_surf_surf_para
 *   src/lib/solverFFT/compute_Lp_Voxels_QS.jl:8-397 compute_Lp_Voxels_QS and its
 *     Integ_vol_vol dispatch, the Lp rows of the Rcc path (compute_rows_Rcc_Lp.jl:20-35),
 *     with that file's integ_line_line_sp (:501-520) and integ_vol_surf (:777-824)
 * Every branch of both dispatches is restated, including the far-field ones that
 * replace a body by a surface, a line or a point once a dimension passes its
 * suppression test (on uniform voxels: centre distances beyond ~200 edges of that
 * dimension), together with their quirks: the 1e-8 nudges of integ_line_point, the
 * origin-dependent collinear line formulas integ_line_line_sp_fft / _P, the 3-term
 * integ_line_surf_ortho_fft and the 4-term integ_surf_surf_ortho_fft. A mode flag
 * turns the suppression off (every entry by its full closed form), which the
 * known-answer tests evaluate in long double as the accurate far-field value.
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
#define ATAN atanl
#define ASINH asinhl
#define FABS fabsl
#define RINT nearbyintl
#define ISFIN isfinite
#else
#define SQRT sqrt
#define LOG log
#define ATAN2 atan2
#define ATAN atan
#define ASINH asinh
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

/* ---------------------------------------------------------------------------------
 * Closed-form primitives of the dispatch. Each returns the signed corner sum and adds
 * sum |term| to *acc. Corner signs: the reference's (-1)^(c1+...+cn [+1]) with 1-based
 * corner indices; with 0-based ones that is (-1)^(sum + n [+1]).
 * --------------------------------------------------------------------------------- */

/* integ_line_point_fft / _P (compute_Lp_Voxels.jl:449-467, compute_row_P_sup.jl:396-414):
 * line x in [x3, x4] at (y3, z3), point (x1, y1, z1) */
static REAL line_point(const REAL* xv, REAL y3, REAL z3, REAL x1, REAL y1, REAL z1, REAL* acc) {
  REAL x3 = xv[0], x4 = xv[1];
  REAL chk = (REAL)1 / (x1 - x3);
  if (isnan(chk) || isinf(chk)) x1 = x1 - (REAL)1e-8;
  chk = (REAL)1 / (x1 - x4);
  if (isnan(chk) || (isinf(chk) && x1 > 0)) x1 = x1 + (REAL)1e-8;
  REAL R1 = SQRT((x1 - x3) * (x1 - x3) + (y1 - y3) * (y1 - y3) + (z1 - z3) * (z1 - z3));
  REAL R2 = SQRT((x1 - x4) * (x1 - x4) + (y1 - y3) * (y1 - y3) + (z1 - z3) * (z1 - z3));
  REAL l1 = LOG((x1 - x3) + R1), l2 = LOG((x1 - x4) + R2);
  REAL Ip = l1 - l2;
  if (!ISFIN(Ip)) {
    l1 = (x1 - x3) / FABS(x1 - x3) * LOG(FABS(x1 - x3));
    l2 = (x1 - x4) / FABS(x1 - x4) * LOG(FABS(x1 - x4));
    Ip = l1 - l2;
  }
  *acc += FABS(l1) + FABS(l2);
  return Ip;
}

/* integ_point_sup_fft / _P (compute_Lp_Voxels.jl:469-489): point, surface in the
 * (x, y) plane at z2. pform 3: integ_point_sup_sharedRis
 * (sharedRis/Song_improved_Ivana_strategy.jl:449-478), whose arctangent takes the
 * quotient, atan(X*Y / (|Z| R)) (NaN when both vanish: the point in the surface's plane,
 * on a corner's line) */
static REAL point_sup(REAL x1, REAL y1, REAL z1, const REAL* x2v, const REAL* y2v, REAL z2,
                      int pform, REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2) {
      REAL X = x1 - x2v[c1], Y = y1 - y2v[c2], Z = z1 - z2;
      REAL R = SQRT(X * X + Y * Y + Z * Z);
      REAL t1 = fin(X * lg(Y + R));
      REAL t2 = fin(Y * lg(X + R));
      REAL t3 = pform == 3 ? -FABS(Z) * ATAN(X * Y / (FABS(Z) * R))
                           : -FABS(Z) * ATAN2(X * Y, FABS(Z) * R);
      sol += sgnp(c1 + c2) * (t1 + t2 + t3);
      *acc += FABS(t1) + FABS(t2) + FABS(t3);
    }
  return sol;
}

/* integ_line_line_sp_fft (compute_Lp_Voxels.jl:514-529) and integ_line_line_sp_P
 * (compute_row_P_sup.jl:461-476), collinear lines. As the reference writes them these
 * take absolute coordinates, not differences; pform 1 selects the _P variant's extra
 * x1*log|x1-x2| term, pform >= 2 the forms that put it inside the (x1-x2)/R factor. */
static REAL ll_sp(const REAL* x1v, const REAL* x2v, int pform, REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2) {
      REAL x1 = x1v[c1], x2 = x2v[c2];
      REAL R = SQRT((x1 - x2) * (x1 - x2));
      REAL t1;
      if (pform >= 2) /* integ_line_line_sp (compute_Lp_Voxels_QS.jl:501-520) and the
                         sharedRis forms (Song_improved_Ivana_strategy.jl:510-532,
                         Song_P_improved_Ivana_strategy.jl:360-382): the x1*log|x1-x2|
                         term inside the (x1-x2)/R factor */
        t1 = (x1 - x2) / R * (x1 - x2 * lg(x2 - x1) + x1 * lg(x1 - x2));
      else {
        t1 = (x1 - x2) / R * (x1 - x2 * lg(x2 - x1));
        if (pform) t1 = t1 + x1 * lg(x1 - x2);
      }
      t1 = fin(t1);
      sol += sgnp(c1 + c2 + 1) * t1;
      *acc += FABS(t1);
    }
  return sol;
}

/* integ_line_line_parall_fft / _P (compute_Lp_Voxels.jl:491-512, compute_row_P_sup.jl:438-459) */
static REAL ll_parall(const REAL* x1v, REAL y1, REAL z1, const REAL* x2v, REAL y2, REAL z2,
                      int pform, REAL* acc) {
  REAL dy = y1 - y2, dz = z1 - z2;
  if (FABS(dy) < (REAL)1e-10 && FABS(dz) < (REAL)1e-10) return ll_sp(x1v, x2v, pform, acc);
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2) {
      REAL X = x1v[c1] - x2v[c2];
      REAL R = SQRT(X * X + dy * dy + dz * dz);
      REAL t1 = fin(X * lg(X + R));
      sol += sgnp(c1 + c2 + 1) * (t1 - R);
      *acc += FABS(t1) + R;
    }
  return sol;
}

/* integ_line_line_ortho_xy_fft / _P (compute_Lp_Voxels.jl:531-551): line along x
 * at (y1, z1), line along y at (x2, z2) */
static REAL ll_ortho(const REAL* x1v, REAL y1, REAL z1, REAL x2, const REAL* y2v, REAL z2,
                     REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2) {
      REAL X = x1v[c1] - x2, Y = y1 - y2v[c2], Z = z1 - z2;
      REAL R = SQRT(X * X + Y * Y + Z * Z);
      REAL t1 = fin(X * lg(Y + R));
      REAL t2 = fin(Y * lg(X + R));
      REAL t3 = -FABS(Z) * ATAN2(X * Y, FABS(Z) * R);
      sol += sgnp(c1 + c2 + 1) * (t1 + t2 + t3);
      *acc += FABS(t1) + FABS(t2) + FABS(t3);
    }
  return sol;
}

/* the six-term triple antiderivative shared by integ_point_vol_fft
 * (compute_Lp_Voxels.jl:553-582) and integ_line_surf_ortho_P (compute_row_P_sup.jl:500-529) */
static REAL f111(REAL X, REAL Y, REAL Z, REAL* acc) {
  REAL R = SQRT(X * X + Y * Y + Z * Z);
  REAL t1 = fin(Y * Z * lg(X + R));
  REAL t2 = fin(X * Z * lg(Y + R));
  REAL t3 = fin(Y * X * lg(Z + R));
  REAL t4 = -(REAL)0.5 * FABS(Z) * Z * ATAN2(X * Y, FABS(Z) * R);
  REAL t5 = -(REAL)0.5 * FABS(Y) * Y * ATAN2(X * Z, FABS(Y) * R);
  REAL t6 = -(REAL)0.5 * FABS(X) * X * ATAN2(Y * Z, FABS(X) * R);
  *acc += FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4) + FABS(t5) + FABS(t6);
  return t1 + t2 + t3 + t4 + t5 + t6;
}

/* integ_point_vol_fft: point, volume */
static REAL point_vol(REAL x1, REAL y1, REAL z1, const REAL* x2v, const REAL* y2v,
                      const REAL* z2v, REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3)
        sol += sgnp(c1 + c2 + c3) * f111(x1 - x2v[c1], y1 - y2v[c2], z1 - z2v[c3], acc);
  return sol;
}

/* integ_line_surf_ortho_fft (compute_Lp_Voxels.jl:584-607; three terms as written there)
 * and integ_line_surf_ortho_P (pform): line along x at (y1, z1), surface in the
 * (y, z) plane at x2 */
static REAL ls_ortho(const REAL* x1v, REAL y1, REAL z1, REAL x2, const REAL* y2v,
                     const REAL* z2v, int pform, REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3) {
        REAL X = x1v[c1] - x2, Y = y1 - y2v[c2], Z = z1 - z2v[c3];
        REAL v;
        if (pform) {
          v = f111(X, Y, Z, acc);
        } else {
          REAL R = SQRT(X * X + Y * Y + Z * Z);
          REAL t1 = fin(Y * Z * lg(X + R));
          REAL t2 = fin(X * Z * lg(Y + R));
          REAL t3 = -FABS(Z) * ATAN2(X * Y, FABS(Z) * R);
          *acc += FABS(t1) + FABS(t2) + FABS(t3);
          v = t1 + t2 + t3;
        }
        sol += sgnp(c1 + c2 + c3 + 1) * v;
      }
  return sol;
}

/* integ_line_surf_para_fft / _P (compute_Lp_Voxels.jl:609-633): surface in the (x, y)
 * plane at z1, line along x at (y2, z2) */
static REAL ls_para(const REAL* x1v, const REAL* y1v, REAL z1, const REAL* x2v, REAL y2, REAL z2,
                    REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3) {
        REAL X = x1v[c1] - x2v[c3], Y = y1v[c2] - y2, Z = z1 - z2;
        REAL R = SQRT(X * X + Y * Y + Z * Z);
        REAL t1 = fin(X * Y * lg(X + R));
        REAL t2 = fin((X * X - Z * Z) / 2 * lg(Y + R));
        REAL t3 = -X * FABS(Z) * ATAN2(X * Y, FABS(Z) * R);
        REAL t4 = -Y / 2 * R;
        sol += sgnp(c1 + c2 + c3 + 3 + 1) * (t1 + t2 + t3 + t4);
        *acc += FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4);
      }
  return sol;
}

/* integ_line_vol_fft (compute_Lp_Voxels.jl:635-668): volume, line along x at (y2, z2) */
static REAL line_vol(const REAL* x1v, const REAL* y1v, const REAL* z1v, const REAL* x2v, REAL y2,
                     REAL z2, REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3)
        for (int c4 = 0; c4 < 2; ++c4) {
          REAL X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2, Z = z1v[c3] - z2;
          REAL R = SQRT(X * X + Y * Y + Z * Z);
          REAL t1 = -(REAL)1 / 3 * Y * Z * R;
          REAL t2 = -(REAL)0.5 * X * FABS(Z) * Z * ATAN2(X * Y, FABS(Z) * R);
          REAL t3 = -(REAL)0.5 * X * FABS(Y) * Y * ATAN2(X * Z, FABS(Y) * R);
          REAL t4 = -(REAL)1 / 6 * (FABS(X) * FABS(X) * FABS(X)) * ATAN2(Y * Z, FABS(X) * R);
          REAL t5 = fin(X * Y * Z * lg(X + R));
          REAL t6 = fin(((REAL)0.5 * (X * X) - (REAL)1 / 6 * (Z * Z)) * Z * lg(Y + R));
          REAL t7 = fin(((REAL)0.5 * (X * X) - (REAL)1 / 6 * (Y * Y)) * Y * lg(Z + R));
          sol += sgnp(c1 + c2 + c3 + c4 + 1) * (t1 + t2 + t3 + t4 + t5 + t6 + t7);
          *acc += FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4) + FABS(t5) + FABS(t6) + FABS(t7);
        }
  return sol;
}

/* integ_surf_surf_para_fft (compute_Lp_Voxels.jl:670-697) = integ_surf_surf_para
 * (compute_Lp_Voxels_QS.jl:695-730): surfaces in (x, y) planes at z1, z2 */
static REAL ss_para(const REAL* x1v, const REAL* y1v, REAL z1, const REAL* x2v, const REAL* y2v,
                    REAL z2, REAL* acc) {
  REAL sol = 0;
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
          *acc += FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4);
        }
  return sol;
}

/* integ_surf_surf_ortho_P (compute_row_P_sup.jl:557-590, seven terms) and, with
 * pform == 0, integ_surf_surf_ortho_fft (compute_Lp_Voxels.jl:699-726, four terms as
 * written there): surface in the (x, y) plane at z1, surface in the (x, z) plane at y2 */
static REAL ss_ortho(const REAL* x1v, const REAL* y1v, REAL z1, const REAL* x2v, REAL y2,
                     const REAL* z2v, int pform, REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3)
        for (int c4 = 0; c4 < 2; ++c4) {
          REAL X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2, Z = z1 - z2v[c3];
          REAL R = SQRT(X * X + Y * Y + Z * Z);
          REAL t1 = -(REAL)1 / 3 * Y * Z * R;
          REAL t2 = -(REAL)0.5 * X * FABS(Z) * Z * ATAN2(X * Y, FABS(Z) * R);
          REAL s, a;
          if (pform) {
            REAL t3 = -(REAL)0.5 * X * FABS(Y) * Y * ATAN2(X * Z, FABS(Y) * R);
            REAL t4 = -(REAL)1 / 6 * FABS(X) * X * X * ATAN2(Y * Z, FABS(X) * R);
            REAL t5 = fin(X * Y * Z * lg(X + R));
            REAL t6 = fin(((REAL)0.5 * X * X - (REAL)1 / 6 * Z * Z) * Z * lg(Y + R));
            REAL t7 = fin(((REAL)0.5 * X * X - (REAL)1 / 6 * Y * Y) * Y * lg(Z + R));
            s = t1 + t2 + t3 + t4 + t5 + t6 + t7;
            a = FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4) + FABS(t5) + FABS(t6) + FABS(t7);
          } else {
            REAL t3 = fin((REAL)0.5 * (X * X - Z * Z) * Y * lg(Y + R));
            REAL t4 = fin((REAL)0.5 * (X * X - Y * Y) * X * lg(X + R));
            s = t1 + t2 + t3 + t4;
            a = FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4);
          }
          sol += sgnp(c1 + c2 + c3 + c4) * s;
          *acc += a;
        }
  return sol;
}

/* integ_vol_surf_fft (compute_Lp_Voxels.jl:728-764) and, with pform 2 or 3,
 * integ_vol_surf (compute_Lp_Voxels_QS.jl:777-824) / integ_vol_surf_sharedRis
 * (Song_improved_Ivana_strategy.jl:818-868), whose second and third terms carry an
 * extra factor (z1 - z2): volume, surface in the (x, y) plane at z2 */
static REAL vol_surf(const REAL* x1v, const REAL* y1v, const REAL* z1v, const REAL* x2v,
                     const REAL* y2v, REAL z2, int pform, REAL* acc) {
  REAL sol = 0;
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2)
      for (int c3 = 0; c3 < 2; ++c3)
        for (int c4 = 0; c4 < 2; ++c4)
          for (int c5 = 0; c5 < 2; ++c5) {
            REAL X = x1v[c1] - x2v[c4], Y = y1v[c2] - y2v[c5], Z = z1v[c3] - z2;
            REAL X2 = X * X, Y2 = Y * Y, Z2 = Z * Z;
            REAL R = SQRT(X2 + Y2 + Z2);
            REAL t1 = (Z2 / 12 - (X2 + Y2) / 8) * Z * R;
            REAL t2 = (pform == 2 || pform == 3) ? fin((Y2 / 2 - Z2 / 6) * X * Z * lg(X + R))
                                 : fin((Y2 / 2 - Z2 / 6) * X * lg(X + R));
            REAL t3 = (pform == 2 || pform == 3) ? fin((X2 / 2 - Z2 / 6) * Y * Z * lg(Y + R))
                                 : fin((X2 / 2 - Z2 / 6) * Y * lg(Y + R));
            REAL t4 = fin((-(X2 * X2) / 24 - (Y2 * Y2) / 24 + (Y2 * X2) / 4) * lg(Z + R));
            REAL t5 = -(FABS(X) * FABS(X) * FABS(X)) * Y / 6 * ATAN2(Y * Z, FABS(X) * R);
            REAL t6 = -X * (FABS(Y) * FABS(Y) * FABS(Y)) / 6 * ATAN2(X * Z, FABS(Y) * R);
            REAL t7 = -X * Y * FABS(Z) * Z / 2 * ATAN2(X * Y, FABS(Z) * R);
            sol += sgnp(c1 + c2 + c3 + c4 + c5 + 5) * (t1 + t2 + t3 + t4 + t5 + t6 + t7);
            *acc += FABS(t1) + FABS(t2) + FABS(t3) + FABS(t4) + FABS(t5) + FABS(t6) + FABS(t7);
          }
  return sol;
}

/* Integ_vol_vol_fft suppression flags (compute_Lp_Voxels.jl:86-172): s1[d] / s2[d] set
 * when dimension d (x, y, z) of voxel 1 / 2 is suppressed */
static void lp_supp(const REAL* x1v, const REAL* y1v, const REAL* z1v, const REAL* x2v,
                    const REAL* y2v, const REAL* z2v, int* s1, int* s2) {
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
  for (int side = 0; side < 2; ++side) {
    REAL a = side ? a2 : a1, b = side ? b2 : b1, c = side ? c2 : c1;
    int* s = side ? s2 : s1;
    s[0] = s[1] = s[2] = 0;
    if (a <= b && a <= c) {
      s[0] = check_fft(e1, e2, e3, V1, V2, dx, min_R, a, b, c);
      if (s[0] && (b > c ? b : c) / (min_R + (REAL)1e-15) < e4) {
        s[1] = check_fft(e1, e2, e3, V1, V2, dy, min_R, b, a, c);
        s[2] = check_fft(e1, e2, e3, V1, V2, dz, min_R, c, a, b);
      }
    } else if (b <= a && b <= c) {
      s[1] = check_fft(e1, e2, e3, V1, V2, dy, min_R, b, a, c);
      if (s[1] && (a > c ? a : c) / (min_R + (REAL)1e-15) < e4) {
        s[0] = check_fft(e1, e2, e3, V1, V2, dx, min_R, a, b, c);
        s[2] = check_fft(e1, e2, e3, V1, V2, dz, min_R, c, a, b);
      }
    } else {
      s[2] = check_fft(e1, e2, e3, V1, V2, dz, min_R, c, a, b);
      if (s[2] && (a > b ? a : b) / (min_R + (REAL)1e-15) < e4) {
        s[0] = check_fft(e1, e2, e3, V1, V2, dx, min_R, a, b, c);
        s[1] = check_fft(e1, e2, e3, V1, V2, dy, min_R, b, a, c);
      }
    }
  }
}

/* The case tree shared by Integ_vol_vol_fft (compute_Lp_Voxels.jl:172-433),
 * Integ_sup_sup_P (compute_row_P_sup.jl:175-379) and Integ_vol_vol
 * (compute_Lp_Voxels_QS.jl:167-393, the Rcc path's Lp dispatcher): the integral of 1/R
 * over two boxes (intervals x1v.., centres xc1.., edge lengths a1..) of which the
 * dimensions flagged in s1 / s2 are collapsed, each collapsed length entering as a
 * factor. The P tree has no volume cases, calls the _P primitives (pform = 1) and passes
 * unit lengths for the face normals. pform = 2 is the Rcc tree: the six-term
 * integ_line_surf_ortho, its own integ_line_line_sp and integ_vol_surf, and in the
 * orthogonal surface-surface case a call whose arguments Julia cannot apply (an
 * interval where the primitive takes a coordinate, compute_Lp_Voxels_QS.jl:330-352):
 * that entry returns NaN and the row driver counts it. pform 3 is the dense RIS Lp tree
 * (Song_improved_Ivana_strategy2, sharedRis/Song_improved_Ivana_strategy.jl:1-404): the
 * Rcc tree's primitives, with the seven-term orthogonal surface-surface form and the
 * one-argument arctangent of integ_point_sup_sharedRis. pform 4 is the dense RIS P tree
 * (Song_P_improved_Ivana_strategy, sharedRis/Song_P_improved_Ivana_strategy.jl:1-256):
 * the _P primitives with the collinear-line form of pform 2. */
static REAL integ_bodies(const REAL* x1v, const REAL* y1v, const REAL* z1v, REAL xc1, REAL yc1,
                         REAL zc1, REAL a1, REAL b1, REAL c1, const REAL* x2v, const REAL* y2v,
                         const REAL* z2v, REAL xc2, REAL yc2, REAL zc2, REAL a2, REAL b2,
                         REAL c2, const int* s1, const int* s2, int pform, REAL* acc) {
  REAL V1 = a1 * b1 * c1, V2 = a2 * b2 * c2;
  int n1 = s1[0] + s1[1] + s1[2], n2 = s2[0] + s2[1] + s2[2];
  int sum = n1 + n2;
  REAL w = 0;
  *acc = 0;
  switch (sum) {
    case 6: { /* point-point */
      REAL d = SQRT((xc1 - xc2) * (xc1 - xc2) + (yc1 - yc2) * (yc1 - yc2) + (zc1 - zc2) * (zc1 - zc2));
      *acc = V1 * V2 / d;
      return V1 * V2 / d;
    }
    case 5: { /* point-line */
      REAL v;
      if (n1 == 3) {
        if (!s2[0]) { w = V1 * V2 / a2; v = line_point(x2v, yc2, zc2, xc1, yc1, zc1, acc); }
        else if (!s2[1]) { w = V1 * V2 / b2; v = line_point(y2v, xc2, zc2, yc1, xc1, zc1, acc); }
        else { w = V1 * V2 / c2; v = line_point(z2v, xc2, yc2, zc1, xc1, yc1, acc); }
      } else {
        if (!s1[0]) { w = V1 * V2 / a1; v = line_point(x1v, yc1, zc1, xc2, yc2, zc2, acc); }
        else if (!s1[1]) { w = V1 * V2 / b1; v = line_point(y1v, xc1, zc1, yc2, xc2, zc2, acc); }
        else { w = V1 * V2 / c1; v = line_point(z1v, xc1, yc1, zc2, xc2, yc2, acc); }
      }
      *acc *= FABS(w);
      return w * v;
    }
    case 4: {
      REAL v;
      if (n1 == 3) { /* point-surface */
        if (s2[0]) { w = V1 * a2; v = point_sup(zc1, yc1, xc1, z2v, y2v, xc2, pform, acc); }
        else if (s2[1]) { w = V1 * b2; v = point_sup(xc1, zc1, yc1, x2v, z2v, yc2, pform, acc); }
        else { w = V1 * c2; v = point_sup(xc1, yc1, zc1, x2v, y2v, zc2, pform, acc); }
      } else if (n2 == 3) {
        if (s1[0]) { w = V2 * a1; v = point_sup(zc2, yc2, xc2, z1v, y1v, xc1, pform, acc); }
        else if (s1[1]) { w = V2 * b1; v = point_sup(xc2, zc2, yc2, x1v, z1v, yc1, pform, acc); }
        else { w = V2 * c1; v = point_sup(xc2, yc2, zc2, x1v, y1v, zc1, pform, acc); }
      } else if (s1[1] && s1[2]) { /* line-line, line 1 along x */
        if (s2[1] && s2[2]) { w = b1 * c1 * b2 * c2; v = ll_parall(x1v, yc1, zc1, x2v, yc2, zc2, pform, acc); }
        else if (s2[0] && s2[2]) { w = b1 * c1 * a2 * c2; v = ll_ortho(x1v, yc1, zc1, xc2, y2v, zc2, acc); }
        else { w = b1 * c1 * a2 * b2; v = ll_ortho(x1v, zc1, yc1, xc2, z2v, yc2, acc); }
      } else if (s1[0] && s1[2]) { /* line 1 along y */
        if (s2[0] && s2[2]) { w = a1 * c1 * a2 * c2; v = ll_parall(y1v, xc1, zc1, y2v, xc2, zc2, pform, acc); }
        else if (s2[0] && s2[1]) { w = a1 * c1 * a2 * b2; v = ll_ortho(y1v, zc1, xc1, yc2, z2v, xc2, acc); }
        else { w = a1 * c1 * b2 * c2; v = ll_ortho(y1v, xc1, zc1, yc2, x2v, zc2, acc); }
      } else { /* line 1 along z */
        if (s2[0] && s2[1]) { w = a1 * b1 * a2 * b2; v = ll_parall(z1v, xc1, yc1, z2v, xc2, yc2, pform, acc); }
        else if (s2[0] && s2[2]) { w = a1 * b1 * a2 * c2; v = ll_ortho(z1v, yc1, xc1, zc2, y2v, xc2, acc); }
        else { w = a1 * b1 * b2 * c2; v = ll_ortho(z1v, xc1, yc1, zc2, x2v, yc2, acc); }
      }
      *acc *= FABS(w);
      return w * v;
    }
    case 3: {
      REAL v;
      if (n1 == 3) { w = a1 * b1 * c1; v = point_vol(xc1, yc1, zc1, x2v, y2v, z2v, acc); }
      else if (n2 == 3) { w = a2 * b2 * c2; v = point_vol(xc2, yc2, zc2, x1v, y1v, z1v, acc); }
      else if (n1 == 1) { /* surface 1, line 2 */
        if (s1[0]) {
          if (!s2[0]) { w = a1 * b2 * c2; v = ls_ortho(x2v, yc2, zc2, xc1, y1v, z1v, pform, acc); }
          else if (!s2[1]) { w = a1 * a2 * c2; v = ls_para(y1v, z1v, xc1, y2v, zc2, xc2, acc); }
          else { w = a1 * a2 * b2; v = ls_para(z1v, y1v, xc1, z2v, yc2, xc2, acc); }
        } else if (s1[1]) {
          if (!s2[0]) { w = b1 * b2 * c2; v = ls_para(x1v, z1v, yc1, x2v, zc2, yc2, acc); }
          else if (!s2[1]) { w = b1 * a2 * c2; v = ls_ortho(y2v, xc2, zc2, yc1, x1v, z1v, pform, acc); }
          else { w = b1 * a2 * b2; v = ls_para(z1v, x1v, yc1, z2v, xc2, yc2, acc); }
        } else {
          if (!s2[0]) { w = c1 * b2 * c2; v = ls_para(x1v, y1v, zc1, x2v, yc2, zc2, acc); }
          else if (!s2[1]) { w = c1 * a2 * c2; v = ls_para(y1v, x1v, zc1, y2v, xc2, zc2, acc); }
          else { w = c1 * a2 * b2; v = ls_ortho(z2v, xc2, yc2, zc1, x1v, y1v, pform, acc); }
        }
      } else { /* surface 2, line 1 */
        if (s2[0]) {
          if (!s1[0]) { w = a2 * b1 * c1; v = ls_ortho(x1v, yc1, zc1, xc2, y2v, z2v, pform, acc); }
          else if (!s1[1]) { w = a2 * a1 * c1; v = ls_para(y2v, z2v, xc2, y1v, zc1, xc1, acc); }
          else { w = a2 * a1 * b1; v = ls_para(z2v, y2v, xc2, z1v, yc1, xc1, acc); }
        } else if (s2[1]) {
          if (!s1[0]) { w = b2 * b1 * c1; v = ls_para(x2v, z2v, yc2, x1v, zc1, yc1, acc); }
          else if (!s1[1]) { w = b2 * a1 * c1; v = ls_ortho(y1v, xc1, zc1, yc2, x2v, z2v, pform, acc); }
          else { w = b2 * a1 * b1; v = ls_para(z2v, x2v, yc2, z1v, xc1, yc1, acc); }
        } else {
          if (!s1[0]) { w = c2 * b1 * c1; v = ls_para(x2v, y2v, zc2, x1v, yc1, zc1, acc); }
          else if (!s1[1]) { w = c2 * a1 * c1; v = ls_para(y2v, x2v, zc2, y1v, xc1, zc1, acc); }
          else { w = c2 * a1 * b1; v = ls_ortho(z1v, xc1, yc1, zc2, x2v, y2v, pform, acc); }
        }
      }
      *acc *= FABS(w);
      return w * v;
    }
    case 2: {
      REAL v;
#define SSO(a, b, c, d, e, f) (pform == 2 ? (REAL)NAN : ss_ortho(a, b, c, d, e, f, pform, acc))
      if (n1 == 2) { /* line 1, volume 2 */
        if (!s1[0]) { w = b1 * c1; v = line_vol(x2v, y2v, z2v, x1v, yc1, zc1, acc); }
        else if (!s1[1]) { w = a1 * c1; v = line_vol(y2v, x2v, z2v, y1v, xc1, zc1, acc); }
        else { w = a1 * b1; v = line_vol(z2v, x2v, y2v, z1v, xc1, yc1, acc); }
      } else if (n2 == 2) {
        if (!s2[0]) { w = b2 * c2; v = line_vol(x1v, y1v, z1v, x2v, yc2, zc2, acc); }
        else if (!s2[1]) { w = a2 * c2; v = line_vol(y1v, x1v, z1v, y2v, xc2, zc2, acc); }
        else { w = a2 * b2; v = line_vol(z1v, x1v, y1v, z2v, xc2, yc2, acc); }
      } else if (s1[0]) { /* surface-surface, surface 1 in the yz plane */
        if (s2[0]) { w = a1 * a2; v = ss_para(y1v, z1v, xc1, y2v, z2v, xc2, acc); }
        else if (s2[1]) { w = a1 * b2; v = SSO(z1v, y1v, xc1, z2v, yc2, x2v); }
        else { w = a1 * c2; v = SSO(y1v, z1v, xc1, y2v, zc2, x2v); }
      } else if (s1[1]) {
        if (s2[0]) { w = b1 * a2; v = SSO(z1v, x1v, yc1, z2v, xc2, y2v); }
        else if (s2[1]) { w = b1 * b2; v = ss_para(x1v, z1v, yc1, x2v, z2v, yc2, acc); }
        else { w = b1 * c2; v = SSO(x1v, z1v, yc1, x2v, zc2, y2v); }
      } else {
        if (s2[0]) { w = c1 * a2; v = SSO(y1v, x1v, zc1, y2v, xc2, z2v); }
        else if (s2[1]) { w = c1 * b2; v = SSO(x1v, y1v, zc1, x2v, yc2, z2v); }
        else { w = c1 * c2; v = ss_para(x1v, y1v, zc1, x2v, y2v, zc2, acc); }
      }
#undef SSO
      *acc *= FABS(w);
      return w * v;
    }
    case 1: {
      REAL v;
      if (s1[0]) { w = a1; v = vol_surf(y2v, z2v, x2v, y1v, z1v, xc1, pform, acc); }
      else if (s1[1]) { w = b1; v = vol_surf(x2v, z2v, y2v, x1v, z1v, yc1, pform, acc); }
      else if (s1[2]) { w = c1; v = vol_surf(x2v, y2v, z2v, x1v, y1v, zc1, pform, acc); }
      else if (s2[0]) { w = a2; v = vol_surf(y1v, z1v, x1v, y2v, z2v, xc2, pform, acc); }
      else if (s2[1]) { w = b2; v = vol_surf(x1v, z1v, y1v, x2v, z2v, yc2, pform, acc); }
      else { w = c2; v = vol_surf(x1v, y1v, z1v, x2v, y2v, zc2, pform, acc); }
      *acc *= FABS(w);
      return w * v;
    }
    default:
      return vol_vol(x1v, y1v, z1v, x2v, y2v, z2v, acc);
  }
}

/* Integ_vol_vol_fft (compute_Lp_Voxels.jl:65-435). *far = 1 when a suppressed branch
 * was taken; suppress == 0 skips the tests (the full volume-volume form). */
static REAL lp_integ(const REAL* x1v, const REAL* y1v, const REAL* z1v, const REAL* x2v,
                     const REAL* y2v, const REAL* z2v, int suppress, int form, REAL* acc,
                     int* far) {
  REAL xc1 = (REAL)0.5 * (x1v[0] + x1v[1]), yc1 = (REAL)0.5 * (y1v[0] + y1v[1]),
       zc1 = (REAL)0.5 * (z1v[0] + z1v[1]);
  REAL xc2 = (REAL)0.5 * (x2v[0] + x2v[1]), yc2 = (REAL)0.5 * (y2v[0] + y2v[1]),
       zc2 = (REAL)0.5 * (z2v[0] + z2v[1]);
  REAL a1 = FABS(x1v[1] - x1v[0]), b1 = FABS(y1v[1] - y1v[0]), c1 = FABS(z1v[1] - z1v[0]);
  REAL a2 = FABS(x2v[1] - x2v[0]), b2 = FABS(y2v[1] - y2v[0]), c2 = FABS(z2v[1] - z2v[0]);
  int s1[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
  if (suppress) lp_supp(x1v, y1v, z1v, x2v, y2v, z2v, s1, s2);
  *far = s1[0] + s1[1] + s1[2] + s2[0] + s2[1] + s2[2] > 0;
  /* the Rcc dispatcher's volume-volume case calls Integ_vol_vol_fft, whose identical
     suppression tests again find nothing collapsed: the same volume-volume closed form */
  return integ_bodies(x1v, y1v, z1v, xc1, yc1, zc1, a1, b1, c1, x2v, y2v, z2v, xc2, yc2, zc2, a2,
                      b2, c2, s1, s2, form, acc);
}

/* One Lp generating row: source centre src, targets centers[N][3] (row-major),
 * current direction dc = 1,2,3. out[k] = 1e-7/S * integral (compute_Lp_Voxels.jl:40-60),
 * scale[k] = the same prefactor times sum|terms|. Returns the count of entries
 * that took a far-field (suppressed) branch. */
static int64_t lp_row_form(int dc, const double* src, const double* centers, int64_t N,
                           double sx_, double sy_, double sz_, int suppress, int form, double* out,
                           double* scale) {
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
    REAL acc;
    int far = 0;
    REAL v = lp_integ(x1v, y1v, z1v, x2v, y2v, z2v, suppress, form, &acc, &far);
    bad += far;
    out[k] = (double)((REAL)1e-7 / S * v);
    if (scale) scale[k] = (double)((REAL)1e-7 / S * acc);
  }
  return bad;
}

int64_t FN(oracle_lp_row)(int dc, const double* src, const double* centers, int64_t N,
                          double sx_, double sy_, double sz_, int suppress, double* out,
                          double* scale) {
  return lp_row_form(dc, src, centers, N, sx_, sy_, sz_, suppress, 0, out, scale);
}

/* compute_Lp_Voxels_QS (compute_Lp_Voxels_QS.jl:8-42), the Rcc path's Lp row: the same
 * driver over the Integ_vol_vol dispatcher (pform 2). Entries in its orthogonal
 * surface-surface case, where the reference raises, come back NaN. */
int64_t FN(oracle_lp_row_qs)(int dc, const double* src, const double* centers, int64_t N,
                             double sx_, double sy_, double sz_, double* out, double* scale) {
  return lp_row_form(dc, src, centers, N, sx_, sy_, sz_, 1, 2, out, scale);
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

/* Integ_sup_sup_P (compute_row_P_sup.jl:106-381): faces given by centre and extents
 * (one extent 0: the face normal). *far = 1 when a suppressed branch was taken. */
static REAL sup_sup(REAL xc1, REAL yc1, REAL zc1, REAL xc2, REAL yc2, REAL zc2, REAL a1, REAL b1,
                    REAL c1, REAL a2, REAL b2, REAL c2, int suppress, REAL* acc, int* far) {
  const REAL e1 = 5e-3, e2 = 1e-3, e3 = 1e-3, e4 = 3e-1;
  REAL x1v[2] = {xc1 - a1 / 2, xc1 + a1 / 2}, y1v[2] = {yc1 - b1 / 2, yc1 + b1 / 2},
       z1v[2] = {zc1 - c1 / 2, zc1 + c1 / 2};
  REAL x2v[2] = {xc2 - a2 / 2, xc2 + a2 / 2}, y2v[2] = {yc2 - b2 / 2, yc2 + b2 / 2},
       z2v[2] = {zc2 - c2 / 2, zc2 + c2 / 2};
  int p1 = 2, p2 = 2; /* normal axis */
  if (a1 <= b1 && a1 <= c1) { p1 = 0; a1 = 1; }
  else if (b1 <= a1 && b1 <= c1) { p1 = 1; b1 = 1; }
  else { c1 = 1; }
  if (a2 <= b2 && a2 <= c2) { p2 = 0; a2 = 1; }
  else if (b2 <= a2 && b2 <= c2) { p2 = 1; b2 = 1; }
  else { c2 = 1; }
  REAL s1 = a1 * b1 * c1, s2 = a2 * b2 * c2;
  int f1[3] = {0, 0, 0}, f2[3] = {0, 0, 0};
  if (suppress) {
    REAL ax[4] = {x1v[0] - x2v[0], x1v[0] - x2v[1], x1v[1] - x2v[0], x1v[1] - x2v[1]};
    REAL ay[4] = {y1v[0] - y2v[0], y1v[0] - y2v[1], y1v[1] - y2v[0], y1v[1] - y2v[1]};
    REAL az[4] = {z1v[0] - z2v[0], z1v[0] - z2v[1], z1v[1] - z2v[0], z1v[1] - z2v[1]};
    REAL mx = minabs4(ax[0], ax[1], ax[2], ax[3]), my = minabs4(ay[0], ay[1], ay[2], ay[3]),
         mz = minabs4(az[0], az[1], az[2], az[3]);
    REAL min_R = SQRT(mx * mx + my * my + mz * mz);
    REAL dx = maxabs4(ax[0], ax[1], ax[2], ax[3]), dy = maxabs4(ay[0], ay[1], ay[2], ay[3]),
         dz = maxabs4(az[0], az[1], az[2], az[3]);
    f1[0] = check_pp(e1, e2, e3, e4, s1, s2, dx, min_R, a1, b1, c1);
    f2[0] = check_pp(e1, e2, e3, e4, s1, s2, dx, min_R, a2, b2, c2);
    f1[1] = check_pp(e1, e2, e3, e4, s1, s2, dy, min_R, b1, a1, c1);
    f2[1] = check_pp(e1, e2, e3, e4, s1, s2, dy, min_R, b2, a2, c2);
    f1[2] = check_pp(e1, e2, e3, e4, s1, s2, dz, min_R, c1, a1, b1);
    f2[2] = check_pp(e1, e2, e3, e4, s1, s2, dz, min_R, c2, a2, b2);
  }
  f1[p1] = 1;
  f2[p2] = 1;
  *far = f1[0] + f1[1] + f1[2] + f2[0] + f2[1] + f2[2] > 2;
  return integ_bodies(x1v, y1v, z1v, xc1, yc1, zc1, a1, b1, c1, x2v, y2v, z2v, xc2, yc2, zc2, a2,
                      b2, c2, f1, f2, 1, acc);
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
                         int suppress, double* out, double* scale) {
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
    int far = 0;
    REAL v = sup_sup(f1[0], f1[1], f1[2], f2[0], f2[1], f2[2], e1[0], e1[1], e1[2], e2[0], e2[1],
                     e2[2], suppress, &acc, &far);
    bad += far;
    /* 1/(4*pi*eps0*A1*d*d) evaluated left to right as the reference writes it */
    REAL pref = (REAL)1 / ((REAL)4 * pi * eps0 * A1 * d2[0] * d2[1]);
    out[k] = (double)((REAL)escal_P * (pref * v));
    if (scale) scale[k] = (double)((REAL)escal_P * (pref * acc));
  }
  return bad;
}

/* ---------------------------------------------------------------------------------
 * Dense RIS fill: sharedRis/calcola_Lp.jl and sharedRis/calcola_P.jl. Bodies are given
 * by their vertex coordinates (a volume: 8 vertices x (x, y, z), volumi[:coordinate];
 * a surface: 4 vertices, superfici["estremi_celle"]), rounded to 14 digits as the
 * reference rounds them (in double in both builds, so that both see the same boxes).
 * --------------------------------------------------------------------------------- */

static double round14d(double v) { return nearbyint(v * 1e14) / 1e14; }

/* isequal, which Julia's unique uses: 0.0 and -0.0 are different values */
static int same_value(REAL a, REAL b) { return a == b && signbit(a) == signbit(b); }

/* calcola_Lp.jl:22-28,43-47: per axis the first and the last entry of
 * unique(round.(coords[[min indices; max indices]], digits=14)), in that order */
static const int RIS_VOL_IDX[3][8] = {{0, 6, 12, 18, 3, 9, 15, 21},
                                      {1, 4, 13, 16, 7, 10, 19, 22},
                                      {2, 5, 8, 11, 14, 17, 20, 23}};

static void ris_vol_box(const double* c24, REAL iv[3][2]) {
  for (int d = 0; d < 3; ++d) {
    REAL v[8];
    for (int i = 0; i < 8; ++i) v[i] = (REAL)round14d(c24[RIS_VOL_IDX[d][i]]);
    REAL last = v[0];
    for (int i = 1; i < 8; ++i) {
      int seen = 0;
      for (int j = 0; j < i; ++j) seen |= same_value(v[i], v[j]);
      if (!seen) last = v[i];
    }
    iv[d][0] = v[0];
    iv[d][1] = last;
  }
}

/* mean_length_rev (sharedRis/Compute_Lp_Self.jl:39-74): distance between the centroids of
 * the two end faces of the brick along curr_dir (1, 2, 3) */
static REAL mean_length_rev(const double* c24, int dir) {
  static const int ends[3][2][4] = {{{0, 2, 4, 6}, {1, 3, 5, 7}},
                                    {{0, 1, 4, 5}, {2, 3, 6, 7}},
                                    {{0, 1, 2, 3}, {4, 5, 6, 7}}};
  REAL d2 = 0;
  for (int k = 0; k < 3; ++k) {
    REAL a = 0, b = 0;
    for (int i = 0; i < 4; ++i) {
      a = a + (REAL)c24[3 * ends[dir - 1][0][i] + k];
      b = b + (REAL)c24[3 * ends[dir - 1][1][i] + k];
    }
    REAL e = (REAL)0.25 * a - (REAL)0.25 * b;
    d2 += e * e;
  }
  return SQRT(d2);
}

/* Compute_Lp_Self (sharedRis/Compute_Lp_Self.jl:1-37), the closed-form self inductance of
 * a rectangular bar of length l, width W, thickness T; 0 when 1/(l W T) is not finite.
 * *mag gets the sum of the magnitudes of its five groups times the prefactor. */
static REAL lp_self(REAL l, REAL W, REAL T, REAL* mag) {
  const REAL pi = 3.14159265358979323846264338327950288L;
  REAL inv = (REAL)1 / (l * W * T);
  *mag = 0;
  if (!ISFIN(inv)) return 0;
  REAL w = W / l, t = T / l;
  REAL r = SQRT(w * w + t * t), aw = SQRT(w * w + 1), at = SQRT(t * t + 1);
  REAL ar = SQRT(w * w + t * t + 1);
  REAL mu0 = 4 * pi * (REAL)1e-7;
  REAL g1 = (REAL)1 / 4 * ((REAL)1 / w * ASINH(w / at) + (REAL)1 / t * ASINH(t / aw) + ASINH((REAL)1 / r));
  REAL g2 = (REAL)1 / 24 *
            (t * t / w * ASINH(w / (t * at * (r + ar))) + w * w / t * ASINH(t / (w * aw * (r + ar))) +
             t * t / (w * w) * ASINH(w * w / (t * r * (at + ar))) +
             w * w / (t * t) * ASINH(t * t / (w * r * (aw + ar))) +
             (REAL)1 / (w * (t * t)) * ASINH(w * (t * t) / (at * (aw + ar))) +
             (REAL)1 / (t * (w * w)) * ASINH(t * (w * w) / (aw * (at + ar))));
  REAL g3 = (REAL)1 / 6 *
            ((REAL)1 / (w * t) * ATAN(w * t / ar) + t / w * ATAN(w / (t * ar)) + w / t * ATAN(t / (w * ar)));
  REAL g4 = (REAL)1 / 60 *
            ((ar + r + t + at) * (t * t) / ((ar + r) * (r + t) * (t + at) * (at + ar)) +
             (ar + r + w + aw) * (w * w) / ((ar + r) * (r + w) * (w + aw) * (aw + ar)) +
             (ar + aw + 1 + at) / ((ar + aw) * (aw + 1) * (1 + at) * (at + ar)));
  REAL g5 = (REAL)1 / 20 * ((REAL)1 / (r + ar) + (REAL)1 / (aw + ar) + (REAL)1 / (at + ar));
  REAL pre = 2 * mu0 * l / pi;
  *mag = FABS(pre) * (FABS(g1) + FABS(g2) + FABS(g3) + FABS(g4) + FABS(g5));
  return pre * (g1 + g2 - g3 - g4 - g5);
}

/* the bar dimensions (l, W, T) Compute_Lp_Self takes for a volume of current direction
 * dir (calcola_Lp.jl:59-77) */
static void ris_lwt(const double* c24, int dir, REAL* l, REAL* W, REAL* T) {
  REAL m1 = FABS(mean_length_rev(c24, 1)), m2 = FABS(mean_length_rev(c24, 2)),
       m3 = FABS(mean_length_rev(c24, 3));
  if (dir == 1) { *l = m1; *W = m3; *T = m2; }
  else if (dir == 2) { *T = m1; *W = m3; *l = m2; }
  else { *W = m1; *l = m3; *T = m2; }
}

double FN(oracle_ris_lp_self)(const double* c24, int dir, double* mag) {
  REAL l, W, T, m;
  ris_lwt(c24, dir, &l, &W, &T);
  REAL v = lp_self(l, W, T, &m);
  if (mag) *mag = (double)m;
  return (double)v;
}

/* One dense Lp block (calculate_Lp_matrix, calcola_Lp.jl:254-306): volumes off .. off+dim-1
 * of coords (24 per volume) with cross-sections S, current direction dir (1, 2, 3).
 * out (dim x dim, column-major, symmetric): 1e-7 / (S_m S_n) * integral * esc off the
 * diagonal (Song_improved_Ivana_strategy2 with suppression), Compute_Lp_Self * esc on
 * it; scale the same prefactors times the sum of |terms|. Returns the count of
 * non-finite entries. */
int64_t FN(oracle_ris_lp_block)(const double* coords, const double* S, int64_t off, int64_t dim,
                                int dir, double esc, double* out, double* scale, int* forms) {
  int64_t bad = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : bad)
  for (int64_t m = 0; m < dim; ++m) {
    const double* cm = coords + 24 * (off + m);
    REAL l, W, T, mag;
    ris_lwt(cm, dir, &l, &W, &T);
    REAL self = lp_self(l, W, T, &mag);
    out[m + m * dim] = (double)(self * (REAL)esc);
    if (scale) scale[m + m * dim] = (double)(mag * FABS((REAL)esc));
    if (!ISFIN(self)) ++bad;
    REAL b1[3][2];
    ris_vol_box(cm, b1);
    for (int64_t n = m + 1; n < dim; ++n) {
      REAL b2[3][2];
      ris_vol_box(coords + 24 * (off + n), b2);
      REAL acc;
      int far = 0;
      REAL v = lp_integ(b1[0], b1[1], b1[2], b2[0], b2[1], b2[2], 1, 3, &acc, &far);
      if (forms) {
        int f1[3], f2[3];
        lp_supp(b1[0], b1[1], b1[2], b2[0], b2[1], b2[2], f1, f2);
        forms[m + n * dim] = forms[n + m * dim] = f1[0] + f1[1] + f1[2] + f2[0] + f2[1] + f2[2];
      }
      REAL pre = (REAL)1e-7 / ((REAL)S[off + m] * (REAL)S[off + n]);
      REAL e = pre * v * (REAL)esc;
      out[m + n * dim] = out[n + m * dim] = (double)e;
      if (scale) scale[m + n * dim] = scale[n + m * dim] = (double)(FABS(pre) * acc * FABS((REAL)esc));
      if (!ISFIN(e)) ++bad;
    }
  }
  return bad;
}

/* process_surfaces! (calcola_P.jl:94-160): the surface's box from vertices 1 and 4,
 * rounded; the normal (the smallest extent) gets length 1 */
static int ris_surf_box(const double* e12, REAL iv[3][2], REAL len[3]) {
  const int lo[3] = {0, 1, 2}, hi[3] = {9, 10, 11};
  for (int d = 0; d < 3; ++d) {
    double a = e12[lo[d]], b = e12[hi[d]];
    iv[d][0] = (REAL)round14d(a < b ? a : b);
    iv[d][1] = (REAL)round14d(a < b ? b : a);
    len[d] = FABS(iv[d][1] - iv[d][0]);
  }
  int nrm = 2;
  if (len[0] <= len[1] && len[0] <= len[2]) nrm = 0;
  else if (len[1] <= len[0] && len[1] <= len[2]) nrm = 1;
  len[nrm] = 1;
  return nrm;
}

/* Song_P_improved_Ivana_strategy (Song_P_improved_Ivana_strategy.jl:1-256) */
static REAL ris_p_integ(REAL iv1[3][2], const REAL* l1, int p1, REAL iv2[3][2], const REAL* l2,
                        int p2, REAL* acc, int* nsum) {
  const REAL e1 = 5e-3, e2 = 1e-3, e3 = 1e-3, e4 = 3e-1;
  REAL s1 = l1[0] * l1[1] * l1[2], s2 = l2[0] * l2[1] * l2[2];
  REAL ax[4] = {iv1[0][0] - iv2[0][0], iv1[0][0] - iv2[0][1], iv1[0][1] - iv2[0][0], iv1[0][1] - iv2[0][1]};
  REAL ay[4] = {iv1[1][0] - iv2[1][0], iv1[1][0] - iv2[1][1], iv1[1][1] - iv2[1][0], iv1[1][1] - iv2[1][1]};
  REAL az[4] = {iv1[2][0] - iv2[2][0], iv1[2][0] - iv2[2][1], iv1[2][1] - iv2[2][0], iv1[2][1] - iv2[2][1]};
  REAL mx = minabs4(ax[0], ax[1], ax[2], ax[3]), my = minabs4(ay[0], ay[1], ay[2], ay[3]),
       mz = minabs4(az[0], az[1], az[2], az[3]);
  REAL min_R = SQRT(mx * mx + my * my + mz * mz);
  REAL dx = maxabs4(ax[0], ax[1], ax[2], ax[3]), dy = maxabs4(ay[0], ay[1], ay[2], ay[3]),
       dz = maxabs4(az[0], az[1], az[2], az[3]);
  int f1[3], f2[3];
  f1[0] = check_pp(e1, e2, e3, e4, s1, s2, dx, min_R, l1[0], l1[1], l1[2]);
  f2[0] = check_pp(e1, e2, e3, e4, s1, s2, dx, min_R, l2[0], l2[1], l2[2]);
  f1[1] = check_pp(e1, e2, e3, e4, s1, s2, dy, min_R, l1[1], l1[0], l1[2]);
  f2[1] = check_pp(e1, e2, e3, e4, s1, s2, dy, min_R, l2[1], l2[0], l2[2]);
  f1[2] = check_pp(e1, e2, e3, e4, s1, s2, dz, min_R, l1[2], l1[0], l1[1]);
  f2[2] = check_pp(e1, e2, e3, e4, s1, s2, dz, min_R, l2[2], l2[0], l2[1]);
  f1[p1] = 1;
  f2[p2] = 1;
  *nsum = f1[0] + f1[1] + f1[2] + f2[0] + f2[1] + f2[2];
  REAL c1[3], c2[3];
  for (int d = 0; d < 3; ++d) {
    c1[d] = (REAL)0.5 * (iv1[d][1] + iv1[d][0]);
    c2[d] = (REAL)0.5 * (iv2[d][1] + iv2[d][0]);
  }
  return integ_bodies(iv1[0], iv1[1], iv1[2], c1[0], c1[1], c1[2], l1[0], l1[1], l1[2], iv2[0],
                      iv2[1], iv2[2], c2[0], c2[1], c2[2], l2[0], l2[1], l2[2], f1, f2, 4, acc);
}

/* The dense P (calculate_P_matrix, calcola_P.jl:162-222): surfaces ends (12 per surface),
 * areas S; out (ns x ns, column-major, symmetric) = integral / (4 pi eps0 S_m S_n) * esc,
 * the diagonal included; scale and forms (2: surface-surface .. 6) as for the Lp block.
 * Returns the count of non-finite entries. */
int64_t FN(oracle_ris_p)(const double* ends, const double* S, int64_t ns, double esc, double* out,
                         double* scale, int* forms) {
  const REAL eps0 = 8.854187816997944e-12L;
  const REAL pi = 3.14159265358979323846264338327950288L;
  int64_t bad = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : bad)
  for (int64_t m = 0; m < ns; ++m) {
    REAL iv1[3][2], l1[3];
    int p1 = ris_surf_box(ends + 12 * m, iv1, l1);
    for (int64_t n = m; n < ns; ++n) {
      REAL iv2[3][2], l2[3];
      int p2 = ris_surf_box(ends + 12 * n, iv2, l2);
      REAL acc;
      int nsum;
      REAL v = ris_p_integ(iv1, l1, p1, iv2, l2, p2, &acc, &nsum);
      if (forms) forms[m + n * ns] = forms[n + m * ns] = nsum;
      REAL inv = (REAL)1 / (4 * pi * eps0 * (REAL)S[m] * (REAL)S[n]);
      REAL e = inv * v * (REAL)esc;
      out[m + n * ns] = out[n + m * ns] = (double)e;
      if (scale) scale[m + n * ns] = scale[n + m * ns] = (double)(FABS(inv) * acc * FABS((REAL)esc));
      if (!ISFIN(e)) ++bad;
    }
  }
  return bad;
}
