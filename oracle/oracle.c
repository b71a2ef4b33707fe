/*
 * oracle.c -- CPU restatement of BookLeaf's per-step hydro path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the checker for the GB300 path.
 * PARITY STATUS: pinned by the reference's Sod known-answer test and by
 * conservation invariants only; bitwise parity with the Fortran serial build
 * is unpinned because no Fortran compiler is available to build it.
 *
 * Each static function restates one reference routine; its comment names
 * the Fortran file and lines it follows.  Arrays keep the reference's
 * 1-based, column-major (NCORN,nel) layout through the E() and C() macros,
 * and the per-phase scratch aliases of src/dataAPI/dataAPI_id.f90:78-111
 * are kept, so that scratch reuse behaves as in the reference.
 *
 * Floating-point conventions: MAX/MIN return the first argument on ties,
 * SIGN(a,b) honours the sign of a negative zero (copysign), integer MOD is
 * C's % for the non-negative operands the reference passes, MODULO is the
 * floored remainder.  Compile with -ffp-contract=off.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define NCORN 4
#define NFACE 4
#define E(a, i) ((a)[(long)(i)-1])
#define C(a, j, i) ((a)[4L * ((long)(i)-1) + (j)-1])

static inline double maxF(double a, double b) { return (b > a) ? b : a; }
static inline double minF(double a, double b) { return (b < a) ? b : a; }
static inline double signF(double a, double b) { return copysign(fabs(a), b); }
static inline int modF(int a, int n) { return a % n; }
static inline int moduloF(int a, int n) { int r = a % n; return (r < 0) ? r + n : r; }

struct orc_ctx {
  bl_sizes s;
  bl_config c;
  void *f[BL_NID + 1];
  unsigned char own[BL_NID + 1];
};

#define R(id) ((double *)ctx->f[id])
#define I(id) ((int *)ctx->f[id])

/* dataAPI_dtstepid_mod (dataAPI_id.f90:78-86) */
#define DT_SCRATCH BL_RSCRATCH11
#define DT_ELLENGTH BL_RSCRATCH12
#define DT_CNU BL_RSCRATCH21
#define DT_CNV BL_RSCRATCH22
#define DT_DU BL_RSCRATCH23
#define DT_DV BL_RSCRATCH24
#define DT_DX BL_RSCRATCH25
#define DT_DY BL_RSCRATCH26
#define DT_STORE BL_RSCRATCH27
/* dataAPI_lagstepid_mod (dataAPI_id.f90:88-98) */
#define LG_CNU BL_RSCRATCH21
#define LG_CNV BL_RSCRATCH22
#define LG_CNFX BL_RSCRATCH23
#define LG_CNFY BL_RSCRATCH24
#define LG_ELENERGY0 BL_RSCRATCH11
#define LG_NDAREA BL_RSCRATCH12
#define LG_NDMASS BL_RSCRATCH13
#define LG_NDUBAR BL_RSCRATCH14
#define LG_NDVBAR BL_RSCRATCH15
#define LG_CPFX BL_RCPSCRATCH21
#define LG_CPFY BL_RCPSCRATCH22
#define LG_CPU BL_RSCRATCH23
#define LG_CPV BL_RSCRATCH24
/* dataAPI_alestepid_mod (dataAPI_id.f90:100-111) */
#define AL_STORE1 BL_RSCRATCH11
#define AL_STORE2 BL_RSCRATCH12
#define AL_STORE3 BL_RSCRATCH13
#define AL_STORE4 BL_RSCRATCH14
#define AL_STORE5 BL_RSCRATCH15
#define AL_STORE6 BL_RSCRATCH16
#define AL_FCDV BL_RSCRATCH21
#define AL_FCDM BL_RSCRATCH22
#define AL_FLUX BL_RSCRATCH23
#define AL_RWORK1 BL_RSCRATCH24
#define AL_RWORK2 BL_RSCRATCH25
#define AL_RWORK3 BL_RSCRATCH26
#define AL_CNU BL_RSCRATCH27
#define AL_CNV BL_RSCRATCH28
#define AL_INDSTATUS BL_ISCRATCH11
#define AL_ZACTIVE BL_ZSCRATCH11

static void set_err(bl_error *e, int ierr, int iout, const char *msg) {
  if (!e) return;
  e->ierr = ierr;
  e->iout = iout;
  strncpy(e->serr, msg ? msg : "", BL_SLEN);
  e->serr[BL_SLEN] = 0;
}

/* ========================= utilities ===================================== */

/* utils_kn_cngather (utils_kn_gather.f90:35-51) */
static void utils_kn_cngather(int n1, const int *indx, const double *aa, double *bb) {
  for (int ii = 1; ii <= n1; ii++)
    for (int jj = 1; jj <= NCORN; jj++) C(bb, jj, ii) = E(aa, C(indx, jj, ii));
}

/* utils_kn_mxgather4 (utils_kn_gather.f90:76-107) */
static void utils_kn_mxgather4(int nmx, const int *imxel, const int *imxfcp, const int *imxncp,
                               const double *e1, const double *e2, const double *e3,
                               const double *e4, double *m1, double *m2, double *m3, double *m4) {
  for (int imx = 1; imx <= nmx; imx++) {
    int iel = E(imxel, imx);
    double w1 = E(e1, iel), w2 = E(e2, iel), w3 = E(e3, iel), w4 = E(e4, iel);
    int icp = E(imxfcp, imx);
    for (int ii = 1; ii <= E(imxncp, imx); ii++) {
      E(m1, icp) = w1; E(m2, icp) = w2; E(m3, icp) = w3; E(m4, icp) = w4;
      icp++;
    }
  }
}

/* utils_kn_mxgathercnav (utils_kn_gather.f90:132-154) */
static void utils_kn_mxgathercnav(int nmx, const int *imxel, const int *imxfcp,
                                  const int *imxncp, const double *el, const double *fr,
                                  double *mx) {
  for (int imx = 1; imx <= nmx; imx++) {
    double w1[NCORN];
    for (int j = 1; j <= NCORN; j++) w1[j - 1] = C(el, j, E(imxel, imx));
    int icp = E(imxfcp, imx);
    for (int ii = 1; ii <= E(imxncp, imx); ii++) {
      for (int j = 1; j <= NCORN; j++) C(mx, j, icp) = E(fr, icp) * w1[j - 1];
      icp++;
    }
  }
}

/* utils_kn_average22 (utils_kn_average.f90:54-81) */
static void utils_kn_average22(int nmx, const int *imxel, const int *imxcp, const int *imxncp,
                               const double *fr, const double *mx1, const double *mx2,
                               double *el1, double *el2) {
  for (int imx = 1; imx <= nmx; imx++) {
    double w1[NCORN] = {0, 0, 0, 0}, w2[NCORN] = {0, 0, 0, 0};
    int icp = E(imxcp, imx);
    for (int ii = 1; ii <= E(imxncp, imx); ii++) {
      for (int j = 1; j <= NCORN; j++) {
        w1[j - 1] = w1[j - 1] + E(fr, icp) * C(mx1, j, icp);
        w2[j - 1] = w2[j - 1] + E(fr, icp) * C(mx2, j, icp);
      }
      icp++;
    }
    int iel = E(imxel, imx);
    for (int j = 1; j <= NCORN; j++) {
      C(el1, j, iel) = w1[j - 1];
      C(el2, j, iel) = w2[j - 1];
    }
  }
}

/* utils_kn_average12 (utils_kn_average.f90:83-107) */
static void utils_kn_average12(int nmx, const int *imxel, const int *imxcp, const int *imxncp,
                               const double *fr, const double *mx1, const double *mx2,
                               double *el) {
  for (int imx = 1; imx <= nmx; imx++) {
    double w1 = 0.0;
    int icp = E(imxcp, imx);
    for (int ii = 1; ii <= E(imxncp, imx); ii++) {
      w1 = w1 + E(fr, icp) * (E(mx1, icp) + E(mx2, icp));
      icp++;
    }
    E(el, E(imxel, imx)) = w1;
  }
}

/* utils_kn_bc (utils_kn_bc.f90:28-58) */
static void utils_kn_bc(int nnd, double rcut, const int *indtype, double *ndu, double *ndv) {
  double w1 = rcut * rcut;
  for (int ind = 1; ind <= nnd; ind++) {
    switch (E(indtype, ind)) {
      case -1: E(ndu, ind) = 0.0; break;
      case -2: E(ndv, ind) = 0.0; break;
      case -3: E(ndu, ind) = 0.0; E(ndv, ind) = 0.0; break;
      default: break;
    }
    double w2 = E(ndu, ind) * E(ndu, ind) + E(ndv, ind) * E(ndv, ind);
    if (w2 < w1) { E(ndu, ind) = 0.0; E(ndv, ind) = 0.0; }
  }
}

/* utils_kn_divide / utils_kn_sum / utils_kn_multiply (utils_kn_math.f90:28-71) */
static void utils_kn_divide(int n, const double *num, const double *den, double *ans) {
  for (int i = 1; i <= n; i++) E(ans, i) = E(num, i) / E(den, i);
}
static void utils_kn_sum(int n, const double *right, double *ans) {
  for (int i = 1; i <= n; i++) E(ans, i) = E(ans, i) + E(right, i);
}
static void utils_kn_multiply(int n, const double *factor, double *ans) {
  for (int i = 1; i <= n; i++) E(ans, i) = E(ans, i) * E(factor, i);
}
/* utils_kn_copy (utils_kn_copy.f90:33-77) */
static void utils_kn_copy(int n, const double *a, double *b) {
  for (int i = 1; i <= n; i++) E(b, i) = E(a, i);
}

/* ========================= geometry ====================================== */

/* geometry_kn_getiso (geometry_kn_volume.f90:30-63) */
static void geometry_kn_getiso(int nel, const double *cnx, const double *cny, double *a1,
                               double *a2, double *a3, double *b1, double *b2, double *b3,
                               double *cnwt) {
  const double ONEBYNINE = 1.0 / 9.0;
  for (int iel = 1; iel <= nel; iel++) {
    double x1 = C(cnx, 1, iel), x2 = C(cnx, 2, iel), x3 = C(cnx, 3, iel), x4 = C(cnx, 4, iel);
    double y1 = C(cny, 1, iel), y2 = C(cny, 2, iel), y3 = C(cny, 3, iel), y4 = C(cny, 4, iel);
    double A1 = 0.25 * (-x1 + x2 + x3 - x4);
    double A2 = 0.25 * (x1 - x2 + x3 - x4);
    double A3 = 0.25 * (-x1 - x2 + x3 + x4);
    double B1 = 0.25 * (-y1 + y2 + y3 - y4);
    double B2 = 0.25 * (y1 - y2 + y3 - y4);
    double B3 = 0.25 * (-y1 - y2 + y3 + y4);
    E(a1, iel) = A1; E(a2, iel) = A2; E(a3, iel) = A3;
    E(b1, iel) = B1; E(b2, iel) = B2; E(b3, iel) = B3;
    C(cnwt, 1, iel) = ONEBYNINE * ((3.0 * B3 - B2) * (3.0 * A1 - A2) - (3.0 * A3 - A2) * (3.0 * B1 - B2));
    C(cnwt, 2, iel) = ONEBYNINE * ((3.0 * B3 + B2) * (3.0 * A1 - A2) - (3.0 * A3 + A2) * (3.0 * B1 - B2));
    C(cnwt, 3, iel) = ONEBYNINE * ((3.0 * B3 + B2) * (3.0 * A1 + A2) - (3.0 * A3 + A2) * (3.0 * B1 + B2));
    C(cnwt, 4, iel) = ONEBYNINE * ((3.0 * B3 - B2) * (3.0 * A1 + A2) - (3.0 * A3 - A2) * (3.0 * B1 + B2));
  }
}

/* geometry_kn_getvolume (geometry_kn_volume.f90:65-79) */
static void geometry_kn_getvolume(int n, const double *a1, const double *a3, const double *b1,
                                  const double *b3, double *vol) {
  for (int ii = 1; ii <= n; ii++) E(vol, ii) = 4.0 * (E(a1, ii) * E(b3, ii) - E(a3, ii) * E(b1, ii));
}

/* geometry_kn_checkvolume (geometry_kn_volume.f90:81-99): the LAST element
 * below val wins. */
static int geometry_kn_checkvolume(int nel, double val, const double *vol) {
  int ierr = BL_SUCCESS;
  for (int iel = 1; iel <= nel; iel++)
    if (E(vol, iel) < val) ierr = -iel;
  return ierr;
}

/* geometry_kn_getfluxvolume (geometry_kn_volume.f90:101-140) */
static void geometry_kn_getfluxvolume(int nel, double cut, const int *ielnd, const double *ndx0,
                                      const double *ndy0, const double *ndx1,
                                      const double *ndy1, double *fcdv) {
  for (long i = 0; i < 4L * nel; i++) fcdv[i] = 0.0;
  for (int iel = 1; iel <= nel; iel++) {
    for (int jj = 1; jj <= NFACE; jj++) {
      int jp = modF(jj, NCORN) + 1;
      int n1 = C(ielnd, jj, iel), n2 = C(ielnd, jp, iel);
      double x1 = E(ndx0, n1), x2 = E(ndx0, n2), y1 = E(ndy0, n1), y2 = E(ndy0, n2);
      double x3 = E(ndx1, n2), x4 = E(ndx1, n1), y3 = E(ndy1, n2), y4 = E(ndy1, n1);
      double a1 = (-x1 - x4) + (x3 + x2);
      double a3 = (-x1 + x4) + (x3 - x2);
      double b1 = (-y1 - y4) + (y3 + y2);
      double b3 = (-y1 + y4) + (y3 - y2);
      C(fcdv, jj, iel) = 0.25 * (a1 * b3 - a3 * b1);
      if (C(fcdv, jj, iel) < cut) C(fcdv, jj, iel) = 0.0;
    }
  }
}

/* geometry_kn_getvertex (geometry_kn_position.f90:28-43) */
static void geometry_kn_getvertex(int nnd, double dt, double *ndx, double *ndy, const double *ndu,
                                  const double *ndv) {
  for (int ind = 1; ind <= nnd; ind++) {
    E(ndx, ind) = E(ndx, ind) + dt * E(ndu, ind);
    E(ndy, ind) = E(ndy, ind) + dt * E(ndv, ind);
  }
}

/* geometry_kn_length helpers (geometry_kn_length.f90:99-139) */
static double geometry_kn_denom(double x1, double y1, double x2, double y2) {
  double w1 = y1 - y2, w2 = x1 - x2;
  return w1 * w1 + w2 * w2;
}
static double geometry_kn_distpp(double x3, double y3, double x4, double y4, double x1, double y1) {
  double w1 = 0.5 * (x3 + x4) - x1;
  double w2 = 0.5 * (y3 + y4) - y1;
  return w1 * w1 + w2 * w2;
}
static double geometry_kn_distpl(double x3, double y3, double x4, double y4, double x1, double y1,
                                 double x2, double y2) {
  double res = 0.5 * (y1 - y2) * (x3 + x4) + 0.5 * (y3 + y4) * (x2 - x1) + y2 * x1 - y1 * x2;
  return res * res;
}

/* geometry_kn_dlm (geometry_kn_length.f90:30-56) */
static void geometry_kn_dlm(const double *x, const double *y, double *res) {
  double x1 = x[0] + x[1], x2 = x[2] + x[3], y1 = y[0] + y[1], y2 = y[2] + y[3];
  x1 = 0.5 * (x1 - x2);
  y1 = 0.5 * (y1 - y2);
  res[0] = x1 * x1 + y1 * y1;
  x1 = x[2] + x[1]; x2 = x[0] + x[3]; y1 = y[2] + y[1]; y2 = y[0] + y[3];
  x1 = 0.5 * (x1 - x2);
  y1 = 0.5 * (y1 - y2);
  res[1] = x1 * x1 + y1 * y1;
  res[2] = res[0];
  res[3] = res[1];
}

/* geometry_kn_dln (geometry_kn_length.f90:58-97) */
static void geometry_kn_dln(const double *x, const double *y, double zcut, double *res) {
  double w1 = geometry_kn_denom(x[2], y[2], x[3], y[3]);
  if (w1 < zcut) res[0] = geometry_kn_distpp(x[0], y[0], x[1], y[1], x[2], y[2]);
  else res[0] = geometry_kn_distpl(x[0], y[0], x[1], y[1], x[2], y[2], x[3], y[3]) / w1;
  w1 = geometry_kn_denom(x[3], y[3], x[0], y[0]);
  if (w1 < zcut) res[1] = geometry_kn_distpp(x[1], y[1], x[2], y[2], x[3], y[3]);
  else res[1] = geometry_kn_distpl(x[1], y[1], x[2], y[2], x[3], y[3], x[0], y[0]) / w1;
  w1 = geometry_kn_denom(x[0], y[0], x[1], y[1]);
  if (w1 < zcut) res[2] = geometry_kn_distpp(x[2], y[2], x[3], y[3], x[0], y[0]);
  else res[2] = geometry_kn_distpl(x[2], y[2], x[3], y[3], x[0], y[0], x[1], y[1]) / w1;
  w1 = geometry_kn_denom(x[1], y[1], x[2], y[2]);
  if (w1 < zcut) res[3] = geometry_kn_distpp(x[3], y[3], x[0], y[0], x[1], y[1]);
  else res[3] = geometry_kn_distpl(x[3], y[3], x[0], y[0], x[1], y[1], x[2], y[2]) / w1;
}

static double minval4(const double *r) {
  double m = r[0];
  for (int i = 1; i < 4; i++) m = minF(m, r[i]);
  return m;
}

/* geometry_kn_getcentroid (geometry_kn_centroid.f90:29-55) */
void orc_centroid(int nvert, const double *xx, const double *yy, double c[2]) {
  double rvol = 0.0;
  c[0] = 0.0; c[1] = 0.0;
  for (int i1 = 1; i1 <= nvert; i1++) {
    int i2 = modF(i1, nvert) + 1;
    double rr = E(xx, i1) * E(yy, i2) - E(xx, i2) * E(yy, i1);
    rvol = rvol + rr;
    c[0] = c[0] + rr * (E(xx, i1) + E(xx, i2));
    c[1] = c[1] + rr * (E(yy, i1) + E(yy, i2));
  }
  rvol = 0.5 * rvol;
  if (rvol > 0.0) { c[0] = c[0] / (6.0 * rvol); c[1] = c[1] / (6.0 * rvol); }
  else { c[0] = 0.0; c[1] = 0.0; }
}

/* geometry_dr_getgeometry (geometry_dr_volume.f90:40-96) */
static int geometry_dr_getgeometry(orc_ctx *ctx) {
  const bl_sizes *s = &ctx->s;
  utils_kn_cngather(s->nel, I(BL_IELND), R(BL_NDX), R(BL_CNX));
  utils_kn_cngather(s->nel, I(BL_IELND), R(BL_NDY), R(BL_CNY));
  geometry_kn_getiso(s->nel, R(BL_CNX), R(BL_CNY), R(BL_A1), R(BL_A2), R(BL_A3), R(BL_B1),
                     R(BL_B2), R(BL_B3), R(BL_CNWT));
  geometry_kn_getvolume(s->nel, R(BL_A1), R(BL_A3), R(BL_B1), R(BL_B3), R(BL_ELVOLUME));
  if (s->ncp > 0) {
    utils_kn_mxgather4(s->nmx, I(BL_IMXEL), I(BL_IMXFCP), I(BL_IMXNCP), R(BL_A1), R(BL_A3),
                       R(BL_B1), R(BL_B3), R(BL_CPA1), R(BL_CPA3), R(BL_CPB1), R(BL_CPB3));
    geometry_kn_getvolume(s->ncp, R(BL_CPA1), R(BL_CPA3), R(BL_CPB1), R(BL_CPB3), R(BL_CPVOLUME));
    utils_kn_multiply(s->ncp, R(BL_FRVOLUME), R(BL_CPVOLUME));
  }
  return geometry_kn_checkvolume(s->nel, 0.0, R(BL_ELVOLUME));
}

/* density_dr_getdensity (density_dr_getdensity.f90:32-46) */
static void density_dr_getdensity(orc_ctx *ctx) {
  utils_kn_divide(ctx->s.nel, R(BL_ELMASS), R(BL_ELVOLUME), R(BL_ELDENSITY));
  if (ctx->s.ncp > 0) utils_kn_divide(ctx->s.ncp, R(BL_CPMASS), R(BL_CPVOLUME), R(BL_CPDENSITY));
}

/* ========================= exp, log, pow ================================= */
/* The equations of state's exp and ** as this project evaluates them: the
   same IEEE operations in the same order as the device's bl_exp, bl_log
   and bl_pow (bookleaf_f90_gb300/csrc/bl_elem.cuh), so that the exact
   device build and this restatement agree bit for bit; the reference's
   gfortran takes these from the C library, which they follow to within
   1-2 units in the last place (tests/test_oracle.py).  exp: Cody-Waite
   reduction by ln 2 (40-bit head) and the Taylor series to r^13; log:
   m 2^e with m in [sqrt(1/2), sqrt(2)), 2 atanh((m-1)/(m+1)) to s^23;
   pow: exp(b log a) with log a and b log a as double-doubles (Dekker's
   product, Knuth's two-sum) carried into exp's reduced argument. */
static double orc_pow2i(int k) { /* 2^k, -1022 <= k <= 1023 */
  uint64_t b = (uint64_t)(k + 1023) << 52;
  double d;
  memcpy(&d, &b, 8);
  return d;
}

static double orc_exp2p(double x, double xl) {
  if (x != x) return x;
  if (x > 709.782712893384) return HUGE_VAL;
  if (x < -745.1332191019412) return 0.0;
  const double kd = nearbyint(x * 1.4426950408889634);
  const double r = ((x - kd * 0.6931471805592082) - kd * 7.371002565167799e-13) + xl;
  double p = 1.6059043836821613e-10;
  p = p * r + 2.08767569878681e-09;
  p = p * r + 2.505210838544172e-08;
  p = p * r + 2.755731922398589e-07;
  p = p * r + 2.7557319223985893e-06;
  p = p * r + 2.48015873015873e-05;
  p = p * r + 0.0001984126984126984;
  p = p * r + 0.001388888888888889;
  p = p * r + 0.008333333333333333;
  p = p * r + 0.041666666666666664;
  p = p * r + 0.16666666666666666;
  p = p * r + 0.5;
  const double q = r + (r * r) * p;
  double e = 1.0 + q;
  int k = (int)kd;
  if (k > 1023) {
    e = e * orc_pow2i(1023);
    k -= 1023;
  } else if (k < -1022) {
    e = e * orc_pow2i(-1022);
    k += 1022;
    if (k < -1022) return 0.0;
  }
  return e * orc_pow2i(k);
}

double orc_exp(double x) { return orc_exp2p(x, 0.0); }

static void orc_two_prod(double a, double b, double *p, double *e) {
  *p = a * b;
  double c = 134217729.0 * a;
  const double ah = c - (c - a), al = a - ah;
  c = 134217729.0 * b;
  const double bh = c - (c - b), bl = b - bh;
  *e = ((ah * bh - *p) + ah * bl + al * bh) + al * bl;
}

static void orc_log_dd(double a, double *hi, double *lo) {
  uint64_t b;
  memcpy(&b, &a, 8);
  int e = 0;
  if ((b >> 52) == 0) {
    a = a * 18014398509481984.0;
    memcpy(&b, &a, 8);
    e = -54;
  }
  e += (int)((b >> 52) & 0x7ff) - 1023;
  uint64_t mb = (b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
  double m;
  memcpy(&m, &mb, 8);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  const double f = m - 1.0;
  const double uh = 2.0 + f, ul = f - (uh - 2.0);
  const double s = f / uh;
  double P, Pe;
  orc_two_prod(s, uh, &P, &Pe);
  const double serr = (((f - P) - Pe) - s * ul) / uh;
  const double s2 = s * s;
  double R = 0.043478260869565216;
  R = R * s2 + 0.047619047619047616;
  R = R * s2 + 0.05263157894736842;
  R = R * s2 + 0.058823529411764705;
  R = R * s2 + 0.06666666666666667;
  R = R * s2 + 0.07692307692307693;
  R = R * s2 + 0.09090909090909091;
  R = R * s2 + 0.1111111111111111;
  R = R * s2 + 0.14285714285714285;
  R = R * s2 + 0.2;
  R = R * s2 + 0.3333333333333333;
  R = R * s2;
  const double t = s + s;
  const double ed = (double)e;
  const double A = ed * 0.6931471805592082;
  const double H = A + t;
  const double bv = H - A;
  const double L1 = (A - (H - bv)) + (t - bv);
  *hi = H;
  *lo = L1 + ((t * R + (serr + serr)) + ed * 7.371002565167799e-13);
}

double orc_log(double a) {
  if (a != a) return a;
  if (a <= 0.0) return a == 0.0 ? -HUGE_VAL : NAN;
  if (a == HUGE_VAL) return a;
  uint64_t b;
  memcpy(&b, &a, 8);
  int e = 0;
  if ((b >> 52) == 0) {
    a = a * 18014398509481984.0;
    memcpy(&b, &a, 8);
    e = -54;
  }
  e += (int)((b >> 52) & 0x7ff) - 1023;
  uint64_t mb = (b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
  double m;
  memcpy(&m, &mb, 8);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  const double f = m - 1.0;
  const double s = f / (2.0 + f);
  const double s2 = s * s;
  double R = 0.043478260869565216;
  R = R * s2 + 0.047619047619047616;
  R = R * s2 + 0.05263157894736842;
  R = R * s2 + 0.058823529411764705;
  R = R * s2 + 0.06666666666666667;
  R = R * s2 + 0.07692307692307693;
  R = R * s2 + 0.09090909090909091;
  R = R * s2 + 0.1111111111111111;
  R = R * s2 + 0.14285714285714285;
  R = R * s2 + 0.2;
  R = R * s2 + 0.3333333333333333;
  R = R * s2;
  const double t = s + s;
  const double ed = (double)e;
  return ed * 0.6931471805592082 + (t + (t * R + ed * 7.371002565167799e-13));
}

double orc_pow(double a, double b) {
  if (b == 0.0 || a == 1.0) return 1.0;
  if (a != a || b != b) return a + b;
  if (a < 0.0) return NAN;
  if (a == 0.0) return b > 0.0 ? 0.0 : HUGE_VAL;
  if (a == HUGE_VAL) return b > 0.0 ? HUGE_VAL : 0.0;
  double lh, ll;
  orc_log_dd(a, &lh, &ll);
  if (fabs(b) > 1e300 || fabs(lh * b) > 1e300) return orc_exp(b * lh);
  double yh, yl;
  orc_two_prod(b, lh, &yh, &yl);
  return orc_exp2p(yh, yl + b * ll);
}

/* ========================= EoS =========================================== */

#define EP(k, m) (cfg->eos_param[(m)][(k)-1])

/* eos_kn_getpressure (eos_kn_forms.f90:28-64) */
static double eos_kn_getpressure(const bl_config *cfg, int mat, double density, double energy) {
  int imat = (mat > 0) ? mat : 0;
  double p, t1, t2, t3, t4, t5;
  switch (cfg->eos_type[imat]) {
    case 0: p = EP(1, imat); break;
    case 1: p = energy * density * (EP(1, imat) - 1.0); break;
    case 2:
      t1 = density / EP(3, imat);
      p = EP(1, imat) * (orc_pow(t1, EP(2, imat)) - 1.0);
      p = maxF(p, EP(4, imat));
      break;
    case 3:
      t1 = EP(4, imat) * EP(6, imat) / density;
      t2 = EP(5, imat) * EP(6, imat) / density;
      t3 = EP(1, imat) * density * energy;
      t4 = (1.0 - EP(1, imat) / t1) * EP(2, imat) * orc_exp(-t1);
      t5 = (1.0 - EP(1, imat) / t2) * EP(3, imat) * orc_exp(-t2);
      p = t3 + t4 + t5;
      break;
    default: p = -1.0; break;
  }
  if (fabs(p) < cfg->pcut) p = 0.0;
  return p;
}

/* eos_kn_getcs2 (eos_kn_forms.f90:66-106) */
static double eos_kn_getcs2(const bl_config *cfg, int mat, double density, double energy) {
  int imat = (mat > 0) ? mat : 0;
  double cs2, t1, t2, t3, t4, t5;
  switch (cfg->eos_type[imat]) {
    case 0: cs2 = cfg->ccut; break;
    case 1: cs2 = EP(1, imat) * (EP(1, imat) - 1.0) * energy; break;
    case 2:
      t1 = density / EP(3, imat);
      t2 = EP(2, imat) - 1.0;
      cs2 = (EP(1, imat) * EP(2, imat)) / EP(3, imat);
      cs2 = cs2 * orc_pow(t1, t2);
      break;
    case 3:
      t1 = EP(6, imat) / density;
      t2 = eos_kn_getpressure(cfg, imat, density, energy);
      t3 = EP(4, imat) * t1;
      t4 = EP(1, imat) / EP(4, imat) + EP(1, imat) * t1 - t3 * t1;
      t4 = t4 * EP(2, imat) * orc_exp(-t3);
      t3 = EP(5, imat) * t1;
      t5 = EP(1, imat) / EP(5, imat) + EP(1, imat) * t1 - t3 * t1;
      t5 = t5 * EP(3, imat) * orc_exp(-t3);
      cs2 = EP(1, imat) * t2 / density + EP(1, imat) * energy - t4 - t5;
      break;
    default: cs2 = cfg->ccut; break;
  }
  cs2 = maxF(cs2, cfg->ccut);
  return cs2;
}

/* eos_kn_geteos (eos_kn_geteos.f90:28-52) */
static void eos_kn_geteos(const bl_config *cfg, int n, const int *imat, const double *density,
                          const double *energy, double *pressure, double *cs2) {
  for (int ii = 1; ii <= n; ii++) {
    E(pressure, ii) = eos_kn_getpressure(cfg, E(imat, ii), E(density, ii), E(energy, ii));
    E(cs2, ii) = eos_kn_getcs2(cfg, E(imat, ii), E(density, ii), E(energy, ii));
  }
}

/* eos_dr_geteos (eos_dr_geteos.f90:35-66) */
static void eos_dr_geteos(orc_ctx *ctx) {
  eos_kn_geteos(&ctx->c, ctx->s.nel, I(BL_IELMAT), R(BL_ELDENSITY), R(BL_ELENERGY),
                R(BL_ELPRESSURE), R(BL_ELCS2));
  if (ctx->s.ncp > 0)
    eos_kn_geteos(&ctx->c, ctx->s.ncp, I(BL_ICPMAT), R(BL_CPDENSITY), R(BL_CPENERGY),
                  R(BL_CPPRESSURE), R(BL_CPCS2));
}

/* ========================= hydro: viscosity ============================== */

/* hydro_kn_initeviscosity (hydro_kn_edgeviscosity.f90:30-71) */
static void hydro_kn_initeviscosity(int nel, const double *cnx, const double *cny,
                                    const double *cnu, const double *cnv, double *elvisc,
                                    double *dx, double *dy, double *du, double *dv,
                                    double *edviscx, double *edviscy) {
  for (int iel = 1; iel <= nel; iel++) {
    E(elvisc, iel) = 0.0;
    for (int j = 1; j <= 4; j++) { C(edviscx, j, iel) = 0.0; C(edviscy, j, iel) = 0.0; }
    for (int j = 1; j <= 4; j++) {
      int jn = modF(j, 4) + 1;
      C(du, j, iel) = C(cnu, jn, iel) - C(cnu, j, iel);
      C(dv, j, iel) = C(cnv, jn, iel) - C(cnv, j, iel);
      C(dx, j, iel) = C(cnx, jn, iel) - C(cnx, j, iel);
      C(dy, j, iel) = C(cny, jn, iel) - C(cny, j, iel);
    }
  }
}

/* hydro_kn_limiteviscosity (hydro_kn_edgeviscosity.f90:73-217) */
static void hydro_kn_limiteviscosity(int nel, double zerocut, double cvisc1, double cvisc2,
                                     const int *indtype, const int *ielel, const int *ielnd,
                                     const int *ielfc, const double *eldensity,
                                     const double *elcs2, const double *du, const double *dv,
                                     const double *dx, const double *dy, double *scratch,
                                     double *edviscx, double *edviscy, double *elvisc) {
  for (int iside = 1; iside <= NFACE / 2; iside++) {
    int is1 = modF(iside + 2, NFACE) + 1;
    int is2 = iside + 1;
    for (int iel = 1; iel <= nel; iel++) {
      int in1 = C(ielel, iside, iel), in2 = C(ielel, iside + 2, iel);
      double w1, w2, w3, w4, den, uhat, vhat, xhat, yhat;
      int ins;
      /* edge 1 */
      w1 = C(du, is1, iel); w2 = C(dv, is1, iel); w3 = C(dx, is1, iel); w4 = C(dy, is1, iel);
      den = sqrt(w1 * w1 + w2 * w2);
      den = 1.0 / maxF(den, zerocut);
      uhat = w1 * den; vhat = w2 * den;
      den = sqrt(w3 * w3 + w4 * w4);
      den = 1.0 / maxF(den, zerocut);
      xhat = w3 * den; yhat = w4 * den;
      den = w3 * xhat + w4 * yhat;
      w1 = (w1 * uhat + w2 * vhat) / signF(maxF(fabs(den), zerocut), den);
      w1 = 1.0 / signF(maxF(fabs(w1), zerocut), w1);
      ins = C(ielfc, iside, iel);
      ins = modF(ins, NFACE) + 1;
      den = C(dx, ins, in1) * xhat + C(dy, ins, in1) * yhat;
      w2 = (C(du, ins, in1) * uhat + C(dv, ins, in1) * vhat) / signF(maxF(fabs(den), zerocut), den);
      C(scratch, 1, iel) = w2 * w1;
      ins = C(ielfc, iside + 2, iel);
      ins = modF(ins + 2, NFACE) + 1;
      den = C(dx, ins, in2) * xhat + C(dy, ins, in2) * yhat;
      w3 = (C(du, ins, in2) * uhat + C(dv, ins, in2) * vhat) / signF(maxF(fabs(den), zerocut), den);
      C(scratch, 2, iel) = w3 * w1;
      /* edge 2 */
      w1 = C(du, is2, iel); w2 = C(dv, is2, iel); w3 = C(dx, is2, iel); w4 = C(dy, is2, iel);
      den = sqrt(w1 * w1 + w2 * w2);
      den = 1.0 / maxF(den, zerocut);
      uhat = w1 * den; vhat = w2 * den;
      den = sqrt(w3 * w3 + w4 * w4);
      den = 1.0 / maxF(den, zerocut);
      xhat = w3 * den; yhat = w4 * den;
      den = w3 * xhat + w4 * yhat;
      w1 = (w1 * uhat + w2 * vhat) / signF(maxF(fabs(den), zerocut), den);
      w1 = 1.0 / signF(maxF(fabs(w1), zerocut), w1);
      ins = C(ielfc, iside, iel);
      ins = modF(ins + 2, NFACE) + 1;
      den = C(dx, ins, in1) * xhat + C(dy, ins, in1) * yhat;
      w2 = (C(du, ins, in1) * uhat + C(dv, ins, in1) * vhat) / signF(maxF(fabs(den), zerocut), den);
      C(scratch, 3, iel) = w2 * w1;
      ins = C(ielfc, iside + 2, iel);
      ins = modF(ins, NFACE) + 1;
      den = C(dx, ins, in2) * xhat + C(dy, ins, in2) * yhat;
      w3 = (C(du, ins, in2) * uhat + C(dv, ins, in2) * vhat) / signF(maxF(fabs(den), zerocut), den);
      C(scratch, 4, iel) = w3 * w1;
    }
    /* BC */
    int insb = iside + 2;
    for (int iel = 1; iel <= nel; iel++) {
      int in1 = C(ielel, iside, iel), in2 = C(ielel, insb, iel);
      if (in1 == iel) {
        int ic1 = C(ielnd, iside, iel), ic2 = C(ielnd, modF(iside, NFACE) + 1, iel);
        if ((E(indtype, ic1) < 0) && (E(indtype, ic2) < 0) && (in2 != iel)) {
          C(scratch, 1, iel) = 1.0; C(scratch, 3, iel) = 1.0;
        } else {
          C(scratch, 1, iel) = 0.0; C(scratch, 3, iel) = 0.0;
        }
      }
      if (in2 == iel) {
        int ic1 = C(ielnd, insb, iel), ic2 = C(ielnd, modF(insb, NFACE) + 1, iel);
        if ((E(indtype, ic1) < 0) && (E(indtype, ic2) < 0) && (in1 != iel)) {
          C(scratch, 2, iel) = 1.0; C(scratch, 4, iel) = 1.0;
        } else {
          C(scratch, 2, iel) = 0.0; C(scratch, 4, iel) = 0.0;
        }
      }
    }
    /* apply limiter */
    for (int iel = 1; iel <= nel; iel++) {
      for (int e = 0; e < 2; e++) {
        int is = e ? is2 : is1;
        int ins = C(ielel, is, iel);
        double w1 = cvisc1 * sqrt(0.5 * (E(elcs2, iel) + E(elcs2, ins)));
        double w2 = C(scratch, e ? 3 : 1, iel);
        double w3 = C(scratch, e ? 4 : 2, iel);
        w2 = minF(minF(minF(0.5 * (w2 + w3), 2.0 * w2), 2.0 * w3), 1.0);
        w2 = maxF(0.0, w2);
        w3 = C(du, is, iel);
        double w4 = C(dv, is, iel);
        w4 = sqrt(w3 * w3 + w4 * w4);
        w3 = 0.5 * (1.0 - w2) * (E(eldensity, iel) + E(eldensity, ins)) * (w1 + cvisc2 * w4);
        C(edviscx, is, iel) = w3;
        C(edviscy, is, iel) = w3;
        w4 = 2.0 * w4 / maxF(E(eldensity, iel), zerocut);
        E(elvisc, iel) = maxF(E(elvisc, iel), w3 * w4);
      }
    }
  }
}

/* hydro_kn_geteviscosity (hydro_kn_edgeviscosity.f90:219-282) */
static void hydro_kn_geteviscosity(int nel, double zerocut, const double *cnx, const double *cny,
                                   const double *cnu, const double *cnv, double *cnviscx,
                                   double *cnviscy) {
  for (int iel = 1; iel <= nel; iel++) {
    double edx[NFACE], edy[NFACE];
    for (int iside = 1; iside <= NFACE; iside++) {
      int ins = modF(iside, NFACE) + 1;
      double w1 = C(cnx, iside, iel), w2 = C(cnx, ins, iel);
      double w3 = 0.5 * (w1 + w2);
      w1 = w2 - w1;
      w2 = 0.25 * (C(cnx, 1, iel) + C(cnx, 2, iel) + C(cnx, 3, iel) + C(cnx, 4, iel));
      double w4 = C(cny, iside, iel), w5 = C(cny, ins, iel);
      double w6 = 0.5 * (w4 + w5);
      w4 = w5 - w4;
      w5 = 0.25 * (C(cny, 1, iel) + C(cny, 2, iel) + C(cny, 3, iel) + C(cny, 4, iel));
      double w7 = sqrt((w2 - w3) * (w2 - w3) + (w5 - w6) * (w5 - w6));
      double w8 = sqrt(w1 * w1 + w4 * w4);
      double den = 1.0 / w7;
      double xhat = (w5 - w6) * den, yhat = (w3 - w2) * den;
      den = 1.0 / w8;
      w1 = w1 * den;
      w2 = w4 * den;
      w3 = xhat * w1 + yhat * w2;
      den = -(signF(1.0, w3) * w7);
      xhat = xhat * den;
      yhat = yhat * den;
      double uhat = C(cnu, ins, iel) - C(cnu, iside, iel);
      double vhat = C(cnv, ins, iel) - C(cnv, iside, iel);
      w5 = sqrt((uhat * uhat) + (vhat * vhat));
      w6 = uhat * xhat + vhat * yhat;
      den = w6 / maxF(w5, zerocut);
      edx[iside - 1] = C(cnviscx, iside, iel) * uhat * den;
      edy[iside - 1] = C(cnviscy, iside, iel) * vhat * den;
      if ((w5 <= zerocut) || (w6 <= zerocut) || (w7 <= zerocut) || (w8 <= zerocut)) {
        edx[iside - 1] = 0.0;
        edy[iside - 1] = 0.0;
      }
    }
    C(cnviscx, 1, iel) = edx[0] - edx[3];
    C(cnviscx, 2, iel) = edx[1] - edx[0];
    C(cnviscx, 3, iel) = edx[2] - edx[1];
    C(cnviscx, 4, iel) = edx[3] - edx[2];
    C(cnviscy, 1, iel) = edy[0] - edy[3];
    C(cnviscy, 2, iel) = edy[1] - edy[0];
    C(cnviscy, 3, iel) = edy[2] - edy[1];
    C(cnviscy, 4, iel) = edy[3] - edy[2];
  }
}

/* hydro_dr_getviscosity (hydro_dr_getviscosity.f90:41-91) */
static void hydro_dr_getviscosity(orc_ctx *ctx) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  if (c->ztq) return; /* the tensor branch of the driver is empty */
  hydro_kn_initeviscosity(s->nel, R(BL_CNX), R(BL_CNY), R(DT_CNU), R(DT_CNV), R(BL_ELVISC),
                          R(DT_DX), R(DT_DY), R(DT_DU), R(DT_DV), R(BL_CNVISCX), R(BL_CNVISCY));
  hydro_kn_limiteviscosity(s->nel, c->zerocut, c->cvisc1, c->cvisc2, I(BL_INDTYPE), I(BL_IELEL),
                           I(BL_IELND), I(BL_IELFC), R(BL_ELDENSITY), R(BL_ELCS2), R(DT_DU),
                           R(DT_DV), R(DT_DX), R(DT_DY), R(DT_STORE), R(BL_CNVISCX),
                           R(BL_CNVISCY), R(BL_ELVISC));
  hydro_kn_geteviscosity(s->nel, c->zerocut, R(BL_CNX), R(BL_CNY), R(DT_CNU), R(DT_CNV),
                         R(BL_CNVISCX), R(BL_CNVISCY));
}

/* hydro_dr_getcs2 (hydro_dr_getcs2.f90:32-44) */
static void hydro_dr_getcs2(orc_ctx *ctx) {
  utils_kn_sum(ctx->s.nel, R(BL_ELVISC), R(BL_ELCS2));
  if (ctx->s.ncp > 0)
    utils_kn_average12(ctx->s.nmx, I(BL_IMXEL), I(BL_IMXFCP), I(BL_IMXNCP), R(BL_FRMASS),
                       R(BL_CPCS2), R(BL_CPVISC), R(BL_ELCS2));
}

/* ========================= hydro: timestep =============================== */

typedef struct {
  double rdt;
  int idt;
  int code;
} dt_cand;

/* hydro_kn_getdtcfl (hydro_kn_getdt.f90:30-85) */
static int hydro_kn_getdtcfl(orc_ctx *ctx, dt_cand *dt) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  const int *ielreg = I(BL_IELREG);
  const double *elcs2 = R(BL_ELCS2), *cnx = R(BL_CNX), *cny = R(BL_CNY);
  double *r11 = R(DT_SCRATCH), *r12 = R(DT_ELLENGTH);
  for (int iel = 1; iel <= s->nel; iel++) {
    int ireg = E(ielreg, iel);
    if (c->zdtnotreg[ireg - 1]) {
      E(r11, iel) = DBL_MAX;
      E(r12, iel) = DBL_MIN;
    } else {
      double res[4], w1;
      if (c->zmidlength[ireg - 1]) geometry_kn_dlm(&C(cnx, 1, iel), &C(cny, 1, iel), res);
      else geometry_kn_dln(&C(cnx, 1, iel), &C(cny, 1, iel), c->zcut, res);
      w1 = minval4(res);
      E(r11, iel) = w1 / E(elcs2, iel);
      E(r12, iel) = w1;
    }
  }
  int ii = 1;
  for (int iel = 2; iel <= s->nel; iel++)
    if (E(r11, iel) < E(r11, ii)) ii = iel;
  double w1 = E(r11, ii);
  if (w1 < 0.0) return BL_FAILURE;
  dt->rdt = c->cfl_sf * sqrt(w1);
  dt->idt = ii;
  dt->code = BL_DT_CFL;
  return BL_SUCCESS;
}

/* hydro_kn_getdtdiv (hydro_kn_getdt.f90:87-122) */
static void hydro_kn_getdtdiv(orc_ctx *ctx, dt_cand *dt) {
  const double *a1 = R(BL_A1), *a3 = R(BL_A3), *b1 = R(BL_B1), *b3 = R(BL_B3);
  const double *vol = R(BL_ELVOLUME), *cnu = R(DT_CNU), *cnv = R(DT_CNV);
  double w2 = DBL_MIN;
  int ii = 0;
  for (int iel = 1; iel <= ctx->s.nel; iel++) {
    double A1 = E(a1, iel), A3 = E(a3, iel), B1 = E(b1, iel), B3 = E(b3, iel);
    double w1 = C(cnu, 1, iel) * (-B3 + B1) + C(cnv, 1, iel) * (A3 - A1) +
                C(cnu, 2, iel) * (B3 + B1) + C(cnv, 2, iel) * (-A3 - A1) +
                C(cnu, 3, iel) * (B3 - B1) + C(cnv, 3, iel) * (-A3 + A1) +
                C(cnu, 4, iel) * (-B3 - B1) + C(cnv, 4, iel) * (A3 + A1);
    w1 = fabs(w1) / E(vol, iel);
    if (w1 > w2) { w2 = w1; ii = iel; }
  }
  dt->rdt = ctx->c.div_sf / w2;
  dt->idt = ii;
  dt->code = BL_DT_DIV;
}

static const char *SDT_NAMES[5] = {" MAXIMUM", "  GROWTH", " INITIAL", "     CFL", "     DIV"};

/* ========================= hydro: forces ================================= */

/* hydro_kn_getforceP (hydro_kn_getforce.f90:30-53) */
static void hydro_kn_getforceP(int n, const double *p, const double *a1, const double *a3,
                               const double *b1, const double *b3, double *fx, double *fy) {
  for (int iel = 1; iel <= n; iel++) {
    double w1 = E(p, iel), A1 = E(a1, iel), A3 = E(a3, iel), B1 = E(b1, iel), B3 = E(b3, iel);
    C(fx, 1, iel) = w1 * (-B3 + B1);
    C(fx, 2, iel) = w1 * (B3 + B1);
    C(fx, 3, iel) = w1 * (B3 - B1);
    C(fx, 4, iel) = w1 * (-B3 - B1);
    C(fy, 1, iel) = w1 * (A3 - A1);
    C(fy, 2, iel) = w1 * (-A3 - A1);
    C(fy, 3, iel) = w1 * (-A3 + A1);
    C(fy, 4, iel) = w1 * (A3 + A1);
  }
}

/* hydro_kn_getforceQ (hydro_kn_getforce.f90:55-71) */
static void hydro_kn_getforceQ(int n, const double *qx, const double *qy, double *fx, double *fy) {
  for (int iel = 1; iel <= n; iel++)
    for (int jj = 1; jj <= NCORN; jj++) {
      C(fx, jj, iel) = C(fx, jj, iel) + C(qx, jj, iel);
      C(fy, jj, iel) = C(fy, jj, iel) + C(qy, jj, iel);
    }
}

/* hydro_kn_getforceHG (hydro_kn_getforce.f90:73-107) */
static void hydro_kn_getforceHG(int nel, double dt, const double *kappareg, const int *ielreg,
                                const double *rho, const double *area, const double *cnu,
                                const double *cnv, double *fx, double *fy) {
  double w4 = 1.0 / dt;
  for (int iel = 1; iel <= nel; iel++) {
    double w2 = C(cnu, 1, iel) - C(cnu, 2, iel) + C(cnu, 3, iel) - C(cnu, 4, iel);
    double w3 = C(cnv, 1, iel) - C(cnv, 2, iel) + C(cnv, 3, iel) - C(cnv, 4, iel);
    int ireg = E(ielreg, iel);
    double w1 = -kappareg[ireg - 1] * E(rho, iel) * E(area, iel) * w4;
    w2 = w1 * w2;
    w3 = w1 * w3;
    C(fx, 1, iel) = C(fx, 1, iel) + w2;
    C(fx, 2, iel) = C(fx, 2, iel) - w2;
    C(fx, 3, iel) = C(fx, 3, iel) + w2;
    C(fx, 4, iel) = C(fx, 4, iel) - w2;
    C(fy, 1, iel) = C(fy, 1, iel) + w3;
    C(fy, 2, iel) = C(fy, 2, iel) - w3;
    C(fy, 3, iel) = C(fy, 3, iel) + w3;
    C(fy, 4, iel) = C(fy, 4, iel) - w3;
  }
}

/* hydro_kn_getforceSP (hydro_kn_getforce.f90:109-188) */
static void hydro_kn_getforceSP(int nel, const double *pmeritreg, const int *ielreg,
                                const double *rho, const double *cs2, const double *cnx,
                                const double *cny, const double *spmass, double *fx,
                                double *fy) {
  for (int iel = 1; iel <= nel; iel++) {
    int ireg = abs(E(ielreg, iel));
    double w1 = pmeritreg[ireg - 1];
    double x3 = 0.25 * (C(cnx, 1, iel) + C(cnx, 2, iel) + C(cnx, 3, iel) + C(cnx, 4, iel));
    double y3 = 0.25 * (C(cny, 1, iel) + C(cny, 2, iel) + C(cny, 3, iel) + C(cny, 4, iel));
    double lfx[NCORN][NCORN], lfy[NCORN][NCORN]; /* lf[j1-1][k-1] = lf(j1,k) */
    for (int j1 = 1; j1 <= NCORN; j1++) {
      double x1 = C(cnx, j1, iel), y1 = C(cny, j1, iel);
      int j2 = modF(j1, NCORN) + 1;
      double x2 = 0.5 * (x1 + C(cnx, j2, iel)), y2 = 0.5 * (y1 + C(cny, j2, iel));
      j2 = modF(j1 + 2, NCORN) + 1;
      double x4 = 0.5 * (x1 + C(cnx, j2, iel)), y4 = 0.5 * (y1 + C(cny, j2, iel));
      double w3 = 0.25 * (-x1 + x2 + x3 - x4);
      double w4 = 0.25 * (-x1 - x2 + x3 + x4);
      double w5 = 0.25 * (-y1 + y2 + y3 - y4);
      double w6 = 0.25 * (-y1 - y2 + y3 + y4);
      double w2 = 4.0 * (w3 * w6 - w4 * w5);
      w2 = C(spmass, j1, iel) / w2;
      w2 = w2 - E(rho, iel);
      w2 = E(cs2, iel) * w2;
      lfx[j1 - 1][0] = w2 * (w5 - w6);
      lfx[j1 - 1][1] = w2 * (w5 + w6);
      lfx[j1 - 1][2] = w2 * (-w5 + w6);
      lfx[j1 - 1][3] = w2 * (-w5 - w6);
      lfy[j1 - 1][0] = w2 * (-w3 + w4);
      lfy[j1 - 1][1] = w2 * (-w3 - w4);
      lfy[j1 - 1][2] = w2 * (w3 - w4);
      lfy[j1 - 1][3] = w2 * (w3 + w4);
    }
#define LF(a, i, k) (a[(i)-1][(k)-1])
    double w2 = 0.5 * (LF(lfx, 1, 4) + LF(lfx, 4, 2));
    double w3 = 0.5 * (LF(lfx, 1, 2) + LF(lfx, 2, 4));
    double w4 = 0.5 * (LF(lfx, 2, 2) + LF(lfx, 3, 4));
    double w5 = 0.5 * (LF(lfx, 4, 4) + LF(lfx, 3, 2));
    double w6 = 0.25 * (LF(lfx, 1, 3) + LF(lfx, 2, 3) + LF(lfx, 3, 3) + LF(lfx, 4, 3));
    C(fx, 1, iel) = C(fx, 1, iel) + w1 * (LF(lfx, 1, 1) + w2 + w3 + w6);
    C(fx, 2, iel) = C(fx, 2, iel) + w1 * (LF(lfx, 2, 1) + w4 + w3 + w6);
    C(fx, 3, iel) = C(fx, 3, iel) + w1 * (LF(lfx, 3, 1) + w4 + w5 + w6);
    C(fx, 4, iel) = C(fx, 4, iel) + w1 * (LF(lfx, 4, 1) + w2 + w5 + w6);
    w2 = 0.5 * (LF(lfy, 1, 4) + LF(lfy, 4, 2));
    w3 = 0.5 * (LF(lfy, 1, 2) + LF(lfy, 2, 4));
    w4 = 0.5 * (LF(lfy, 2, 2) + LF(lfy, 3, 4));
    w5 = 0.5 * (LF(lfy, 4, 4) + LF(lfy, 3, 2));
    w6 = 0.25 * (LF(lfy, 1, 3) + LF(lfy, 2, 3) + LF(lfy, 3, 3) + LF(lfy, 4, 3));
    C(fy, 1, iel) = C(fy, 1, iel) + w1 * (LF(lfy, 1, 1) + w2 + w3 + w6);
    C(fy, 2, iel) = C(fy, 2, iel) + w1 * (LF(lfy, 2, 1) + w4 + w3 + w6);
    C(fy, 3, iel) = C(fy, 3, iel) + w1 * (LF(lfy, 3, 1) + w4 + w5 + w6);
    C(fy, 4, iel) = C(fy, 4, iel) + w1 * (LF(lfy, 4, 1) + w2 + w5 + w6);
#undef LF
  }
}

/* hydro_dr_getforce (hydro_dr_getforce.f90:40-91) */
static void hydro_dr_getforce(orc_ctx *ctx, const bl_timestep *ts) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  hydro_kn_getforceP(s->nel, R(BL_ELPRESSURE), R(BL_A1), R(BL_A3), R(BL_B1), R(BL_B3),
                     R(LG_CNFX), R(LG_CNFY));
  if (s->ncp > 0)
    hydro_kn_getforceP(s->ncp, R(BL_CPPRESSURE), R(BL_CPA1), R(BL_CPA3), R(BL_CPB1),
                       R(BL_CPB3), R(LG_CPFX), R(LG_CPFY));
  hydro_kn_getforceQ(s->nel, R(BL_CNVISCX), R(BL_CNVISCY), R(LG_CNFX), R(LG_CNFY));
  if (s->ncp > 0)
    hydro_kn_getforceQ(s->ncp, R(BL_CPVISCX), R(BL_CPVISCY), R(LG_CPFX), R(LG_CPFY));
  if (c->zsp)
    hydro_kn_getforceSP(s->nel, c->pmeritreg, I(BL_IELREG), R(BL_ELDENSITY), R(BL_ELCS2),
                        R(BL_CNX), R(BL_CNY), R(BL_SPMASS), R(LG_CNFX), R(LG_CNFY));
  if (ts->zcorrector && c->zhg)
    hydro_kn_getforceHG(s->nel, ts->dt, c->kappareg, I(BL_IELREG), R(BL_ELDENSITY),
                        R(BL_ELVOLUME), R(LG_CNU), R(LG_CNV), R(LG_CNFX), R(LG_CNFY));
}

/* ========================= hydro: acceleration =========================== */

/* hydro_kn_scatteracceleration (hydro_kn_getacceleration.f90:30-74) */
static void hydro_kn_scatteracceleration(int nel, int nnd, double zerocut, const int *ielsort,
                                         const int *ielnd, const double *rho,
                                         const double *cnwt, const double *cnmass,
                                         double *ndarea, double *ndmass, const double *cnfx,
                                         const double *cnfy, double *ndudot, double *ndvdot) {
  for (int ind = 1; ind <= nnd; ind++) {
    E(ndmass, ind) = 0.0; E(ndarea, ind) = 0.0; E(ndudot, ind) = 0.0; E(ndvdot, ind) = 0.0;
  }
  for (int jj = 1; jj <= NCORN; jj++) {
    for (int kk = 1; kk <= nel; kk++) {
      int iel = E(ielsort, kk);
      int ind = C(ielnd, jj, iel);
      if (C(cnmass, jj, iel) > zerocut) {
        E(ndmass, ind) = E(ndmass, ind) + C(cnmass, jj, iel);
      } else {
        int ii = jj - 1;
        if (ii == 0) ii = 4;
        if (C(cnmass, ii, iel) > zerocut) E(ndmass, ind) = E(ndmass, ind) + C(cnmass, ii, iel);
        else E(ndmass, ind) = E(ndmass, ind) + E(rho, iel) * C(cnwt, jj, iel);
      }
      E(ndarea, ind) = E(ndarea, ind) + C(cnwt, jj, iel);
      E(ndudot, ind) = E(ndudot, ind) + C(cnfx, jj, iel);
      E(ndvdot, ind) = E(ndvdot, ind) + C(cnfy, jj, iel);
    }
  }
}

/* hydro_kn_getacceleration (hydro_kn_getacceleration.f90:76-100) */
static void hydro_kn_getacceleration(int nnd, double dencut, double zerocut, const double *ndarea,
                                     double *ndmass, double *ndudot, double *ndvdot) {
  for (int ind = 1; ind <= nnd; ind++) {
    double w1 = dencut * E(ndarea, ind);
    if (E(ndmass, ind) > w1) {
      E(ndudot, ind) = E(ndudot, ind) / E(ndmass, ind);
      E(ndvdot, ind) = E(ndvdot, ind) / E(ndmass, ind);
    } else {
      E(ndudot, ind) = 0.0;
      E(ndvdot, ind) = 0.0;
      E(ndmass, ind) = maxF(zerocut, w1);
    }
  }
}

/* hydro_kn_applyacceleration (hydro_kn_getacceleration.f90:102-122) */
static void hydro_kn_applyacceleration(int nnd, double dt, double *ubar, double *vbar, double *u,
                                       double *v) {
  double dt05 = 0.5 * dt;
  for (int ind = 1; ind <= nnd; ind++) {
    double w1 = E(u, ind), w2 = E(v, ind);
    E(u, ind) = w1 + dt * E(ubar, ind);
    E(v, ind) = w2 + dt * E(vbar, ind);
    E(ubar, ind) = w1 + dt05 * E(ubar, ind);
    E(vbar, ind) = w2 + dt05 * E(vbar, ind);
  }
}

/* inf_solver_getacceleration (inf_solver_getacceleration.f90:35-66) */
static void inf_solver_getacceleration(orc_ctx *ctx, const bl_timestep *ts) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  /* hydro_dr_initacceleration (hydro_dr_getacceleration.f90:61-79) */
  if (s->ncp > 0)
    utils_kn_average22(s->nmx, I(BL_IMXEL), I(BL_IMXFCP), I(BL_IMXNCP), R(BL_FRVOLUME),
                       R(LG_CPFX), R(LG_CPFY), R(LG_CNFX), R(LG_CNFY));
  /* hydro_dr_scatteracceleration (:81-97) */
  hydro_kn_scatteracceleration(s->nel1, s->nnd1, c->zerocut, I(BL_IELSORT1), I(BL_IELND),
                               R(BL_ELDENSITY), R(BL_CNWT), R(BL_CNMASS), R(LG_NDAREA),
                               R(LG_NDMASS), R(LG_CNFX), R(LG_CNFY), R(LG_NDUBAR),
                               R(LG_NDVBAR));
  /* hydro_dr_getacceleration (:44-59) */
  hydro_kn_getacceleration(s->nnd, c->dencut, c->zerocut, R(LG_NDAREA), R(LG_NDMASS),
                           R(LG_NDUBAR), R(LG_NDVBAR));
  utils_kn_bc(s->nnd, c->accut, I(BL_INDTYPE), R(LG_NDUBAR), R(LG_NDVBAR));
  /* hydro_dr_applyacceleration (:99-112) */
  hydro_kn_applyacceleration(s->nnd, ts->dt, R(LG_NDUBAR), R(LG_NDVBAR), R(BL_NDU), R(BL_NDV));
  utils_kn_cngather(s->nel, I(BL_IELND), R(LG_NDUBAR), R(LG_CNU));
  utils_kn_cngather(s->nel, I(BL_IELND), R(LG_NDVBAR), R(LG_CNV));
}

/* ========================= hydro: energy ================================= */

/* hydro_kn_getenergy (hydro_kn_getenergy.f90:29-52) */
static void hydro_kn_getenergy(int n, double dt, double zerocut, double *e, const double *m,
                               const double *fx, const double *fy, const double *u,
                               const double *v) {
  for (int iel = 1; iel <= n; iel++) {
    double w1 = C(fx, 1, iel) * C(u, 1, iel) + C(fy, 1, iel) * C(v, 1, iel) +
                C(fx, 2, iel) * C(u, 2, iel) + C(fy, 2, iel) * C(v, 2, iel) +
                C(fx, 3, iel) * C(u, 3, iel) + C(fy, 3, iel) * C(v, 3, iel) +
                C(fx, 4, iel) * C(u, 4, iel) + C(fy, 4, iel) * C(v, 4, iel);
    w1 = -(w1 / maxF(E(m, iel), zerocut));
    E(e, iel) = E(e, iel) + w1 * dt;
  }
}

/* hydro_dr_getenergy (hydro_dr_getenergy.f90:35-64) */
static void hydro_dr_getenergy(orc_ctx *ctx, const bl_timestep *ts) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  hydro_kn_getenergy(s->nel, ts->dts, c->zerocut, R(BL_ELENERGY), R(BL_ELMASS), R(LG_CNFX),
                     R(LG_CNFY), R(LG_CNU), R(LG_CNV));
  if (s->ncp > 0) {
    utils_kn_mxgathercnav(s->nmx, I(BL_IMXEL), I(BL_IMXFCP), I(BL_IMXNCP), R(LG_CNU),
                          R(BL_FRVOLUME), R(LG_CPU));
    utils_kn_mxgathercnav(s->nmx, I(BL_IMXEL), I(BL_IMXFCP), I(BL_IMXNCP), R(LG_CNV),
                          R(BL_FRVOLUME), R(LG_CPV));
    hydro_kn_getenergy(s->ncp, ts->dts, c->zerocut, R(BL_CPENERGY), R(BL_CPMASS), R(LG_CPFX),
                       R(LG_CPFY), R(LG_CPU), R(LG_CPV));
  }
}

/* ========================= time ========================================== */

static void time_set_sdt(bl_timestep *ts, int code) {
  memset(ts->sdt, 0, sizeof(ts->sdt));
  memcpy(ts->sdt, SDT_NAMES[code], 8);
}

/* time_dr_setmaterial (time_dr_advance.f90:134-155) */
static void time_set_mdt(orc_ctx *ctx, bl_timestep *ts) {
  memset(ts->mdt, 0, sizeof(ts->mdt));
  if (ts->idtel > 0) {
    int ii = E(I(BL_IELMAT), ts->idtel);
    if (ii > 0) { ts->imdt = ii; snprintf(ts->mdt, sizeof(ts->mdt), "%10d", ii); }
    else { ts->imdt = 0; memcpy(ts->mdt, "     MIXED", 10); }
  } else {
    ts->imdt = -1;
    memcpy(ts->mdt, "   UNKNOWN", 10);
  }
}

/* ========================= ALE =========================================== */

/* ale_kn_updatebasisel (ale_kn_advect.f90:31-61) */
static void ale_kn_updatebasisel(int nel, double zerocut, double dencut, const double *totv,
                                 const double *totm, double *cutv, double *cutm, double *elvpr,
                                 double *elmpr, double *eldpr, double *elv, double *elm,
                                 double *eld) {
  for (int iel = 1; iel <= nel; iel++) {
    E(elvpr, iel) = E(elv, iel);
    E(elmpr, iel) = E(elm, iel);
    E(eldpr, iel) = E(eld, iel);
    E(cutv, iel) = zerocut;
    E(cutm, iel) = E(elvpr, iel) * dencut;
    E(elv, iel) = E(elv, iel) + E(totv, iel);
    E(elm, iel) = E(elm, iel) + E(totm, iel);
    E(eld, iel) = E(elm, iel) / E(elv, iel);
  }
}

/* ale_kn_initbasisnd (ale_kn_advect.f90:63-78) */
static void ale_kn_initbasisnd(int nnd, double *v0, double *v1, double *m0) {
  for (int ind = 1; ind <= nnd; ind++) { E(v0, ind) = 0.0; E(v1, ind) = 0.0; E(m0, ind) = 0.0; }
}

/* ale_kn_calcbasisnd (ale_kn_advect.f90:80-126) */
static void ale_kn_calcbasisnd(int nel, const int *ielnd, const int *ielsort, const double *elv0,
                               const double *elv1, const double *cnm1, double *ndv0,
                               double *ndv1, double *ndm0, double *cnm0) {
  for (int ii = 1; ii <= nel; ii++) {
    int iel = E(ielsort, ii);
    double w1 = 0.25 * E(elv0, iel), w2 = 0.25 * E(elv1, iel);
    for (int j = 1; j <= NCORN; j++) {
      double w3 = C(cnm1, j, iel);
      C(cnm0, j, iel) = w3;
      int ind = C(ielnd, j, iel);
      E(ndv0, ind) = E(ndv0, ind) + w1;
      E(ndv1, ind) = E(ndv1, ind) + w2;
      E(ndm0, ind) = E(ndm0, ind) + w3;
    }
  }
}

/* ale_kn_fluxbasisnd (ale_kn_advect.f90:128-188) */
static void ale_kn_fluxbasisnd(int id1, int id2, int nel, const int *ielel, const int *ielsd,
                               const int *ielsort, const double *fcdv, const double *fcdm,
                               double *cndv, double *cndm, double *cnflux) {
  for (int iel = 1; iel <= nel; iel++)
    for (int j = 1; j <= NCORN; j++) C(cnflux, j, iel) = 0.0;
  for (int i1 = id1; i1 <= id2; i1++) {
    int i2 = i1 + 2;
    for (int ii = 1; ii <= nel; ii++) {
      int iel = E(ielsort, ii);
      int ie1 = C(ielel, i1, iel), ie2 = C(ielel, i2, iel);
      int is1 = C(ielsd, i1, iel), is2 = C(ielsd, i2, iel);
      double w1 = C(fcdv, is1, ie1), w2 = C(fcdv, is2, ie2);
      double w3 = C(fcdm, is1, ie1), w4 = C(fcdm, is2, ie2);
      if (ie1 == iel) { w1 = 0.0; w3 = 0.0; }
      if (ie2 == iel) { w2 = 0.0; w4 = 0.0; }
      w1 = w1 - C(fcdv, i1, iel);
      w2 = w2 - C(fcdv, i2, iel);
      w1 = 0.25 * (w1 - w2);
      C(cndv, i1, iel) = w1;
      C(cndv, i2, iel) = w1;
      w1 = w3 - C(fcdm, i1, iel);
      w2 = w4 - C(fcdm, i2, iel);
      w3 = 0.25 * (w1 - w2);
      C(cndm, i1, iel) = w3;
      C(cndm, i2, iel) = w3;
      w3 = 0.25 * (w1 + w2);
      for (int j = 1; j <= NCORN; j++) C(cnflux, j, iel) = C(cnflux, j, iel) + w3;
    }
  }
}

/* ale_kn_massbasisnd (ale_kn_advect.f90:190-219) */
static void ale_kn_massbasisnd(int nel, const int *ielnd, const int *ielsort, const double *cnflux,
                               double *cnm1, double *ndm1) {
  for (int ii = 1; ii <= nel; ii++) {
    int iel = E(ielsort, ii);
    for (int j = 1; j <= NCORN; j++) C(cnm1, j, iel) = C(cnm1, j, iel) + C(cnflux, j, iel);
    for (int j = 1; j <= NCORN; j++) {
      int ind = C(ielnd, j, iel);
      E(ndm1, ind) = E(ndm1, ind) + C(cnflux, j, iel);
    }
  }
}

/* ale_kn_cutbasisnd (ale_kn_advect.f90:221-237) */
static void ale_kn_cutbasisnd(int nnd, double cut, double dencut, const double *ndv0, double *cutv,
                              double *cutm) {
  for (int ind = 1; ind <= nnd; ind++) { E(cutv, ind) = cut; E(cutm, ind) = dencut * E(ndv0, ind); }
}

/* ale_kn_activend (ale_kn_advect.f90:239-258) */
static void ale_kn_activend(int nnd, int ibc, const int *indstatus, const int *indtype,
                            int *zactive) {
  for (int ind = 1; ind <= nnd; ind++)
    E(zactive, ind) = (E(indstatus, ind) > 0) && (E(indtype, ind) != ibc) && (E(indtype, ind) != -3);
}

/* ale_kn_fluxelvl (ale_kn_advectors.f90:30-81) */
static void ale_kn_fluxelvl(int id1, int id2, int nel, const int *ielel, const int *ielfc,
                            const double *cnbasis, const double *fcdbasis, const double *elvar,
                            double *fcflux) {
  for (long i = 0; i < 4L * nel; i++) fcflux[i] = 0.0;
  for (int i1 = id1; i1 <= id2; i1++) {
    int i2 = i1 + 2;
    for (int iel = 1; iel <= nel; iel++) {
      int iel2 = C(ielel, i2, iel);
      int j2 = C(ielfc, i2, iel);
      int j1 = modF(i2, NCORN) + 1;
      double r3 = C(cnbasis, i2, iel) + C(cnbasis, j1, iel);
      j1 = modF(j2, NCORN) + 1;
      double w5 = r3 + C(cnbasis, j2, iel2) + C(cnbasis, j1, iel2);
      int iel1 = C(ielel, i1, iel);
      j2 = C(ielfc, i1, iel);
      j1 = i1 + 1;
      double r4 = C(cnbasis, i1, iel) + C(cnbasis, j1, iel);
      j1 = modF(j2, NCORN) + 1;
      double w6 = r4 + C(cnbasis, j2, iel1) + C(cnbasis, j1, iel1);
      double rv = E(elvar, iel);
      double r1 = C(fcdbasis, i1, iel), r2 = C(fcdbasis, i2, iel);
      double w1 = rv - E(elvar, iel2);
      double w2 = E(elvar, iel1) - rv;
      double w3 = fabs(w1), w4 = fabs(w2);
      double w7 = signF(1.0, w2);
      double w8 = (w1 * w6 * w6 + w2 * w5 * w5) / (w5 * w6 * (w5 + w6));
      double grad = w7 * minF(minF(fabs(w8), w3 / w5), w4 / w6);
      if (w1 * w2 <= 0.0) grad = 0.0;
      r1 = r1 * (rv + grad * (r3 - 0.5 * r1));
      r2 = r2 * (rv - grad * (r4 - 0.5 * r2));
      C(fcflux, i1, iel) = r1;
      C(fcflux, i2, iel) = r2;
    }
  }
}

/* ale_kn_fluxndvl (ale_kn_advectors.f90:83-153) */
static void ale_kn_fluxndvl(int nel, const int *ielel, const int *ielfc, const double *cnbasis,
                            const double *cndbasis, const double *cnvar, double *cnflux) {
  for (long i = 0; i < 4L * nel; i++) cnflux[i] = 0.0;
  for (int ilfcl = 1; ilfcl <= 2; ilfcl++) {
    int ilfcr = ilfcl + 2;
    for (int icn = 1; icn <= 2; icn++) {
      int ilndl = ilfcl + icn - 1;
      int ilndr = modF(ilfcr - icn + 1, NCORN) + 1;
      for (int iel = 1; iel <= nel; iel++) {
        double rd = 0.0;
        int iell = C(ielel, ilfcl, iel), ielr = C(ielel, ilfcr, iel);
        int ifcl = C(ielfc, ilfcl, iel), ifcr = C(ielfc, ilfcr, iel);
        int ii = ilfcl + 2 * (icn - 1);
        if (C(cndbasis, ii, iel) > 0.0) {
          int ilnndl = modF(ifcl + icn, NCORN) + 1;
          int ilnndr = modF(ifcl - icn + 1, NCORN) + 1;
          double rv = C(cnvar, ilndl, iel);
          rd = C(cnbasis, ilndl, iel) - 0.5 * C(cndbasis, ii, iel);
          double w5 = C(cnbasis, ilndl, iel) + C(cnbasis, ilndr, iel);
          double w6 = C(cnbasis, ilnndl, iell) + C(cnbasis, ilnndr, iell);
          double w1 = rv - C(cnvar, ilnndl, iell);
          double w2 = C(cnvar, ilndr, iel) - rv;
          double w3 = fabs(w1), w4 = fabs(w2);
          double w7 = signF(1.0, w2);
          double w8 = (w2 * w6 * w6 + w1 * w5 * w5) / (w5 * w6 * (w5 + w6));
          double grad = w7 * minF(minF(fabs(w8), w3 / w6), w4 / w5);
          if (w1 * w2 <= 0.0) grad = 0.0;
          rd = C(cndbasis, ii, iel) * (rv + grad * rd);
        }
        if (C(cndbasis, ii, iel) < 0.0) {
          int ilnndl = modF(ifcr + icn - 2, NCORN) + 1;
          int ilnndr = moduloF(ifcr - icn - 1, NCORN) + 1;
          double rv = C(cnvar, ilndr, iel);
          rd = C(cnbasis, ilndr, iel) + 0.5 * C(cndbasis, ii, iel);
          double w5 = C(cnbasis, ilndl, iel) + C(cnbasis, ilndr, iel);
          double w6 = C(cnbasis, ilnndl, ielr) + C(cnbasis, ilnndr, ielr);
          double w1 = rv - C(cnvar, ilndl, iel);
          double w2 = C(cnvar, ilnndr, ielr) - rv;
          double w3 = fabs(w1), w4 = fabs(w2);
          double w7 = signF(1.0, w2);
          double w8 = (w1 * w6 * w6 + w2 * w5 * w5) / (w5 * w6 * (w5 + w6));
          double grad = -(w7 * minF(minF(fabs(w8), w3 / w5), w4 / w6));
          if (w1 * w2 <= 0.0) grad = 0.0;
          rd = C(cndbasis, ii, iel) * (rv + grad * rd);
        }
        C(cnflux, ilndl, iel) = C(cnflux, ilndl, iel) - rd;
        C(cnflux, ilndr, iel) = C(cnflux, ilndr, iel) + rd;
      }
    }
  }
}

/* ale_kn_sumflux (ale_kn_advectors.f90:216-244) */
static void ale_kn_sumflux(int id1, int id2, int nel, const int *ielel, const int *ielfc,
                           const double *fcflux, double *elflux) {
  for (int iel = 1; iel <= nel; iel++) E(elflux, iel) = 0.0;
  for (int i1 = id1; i1 <= id2; i1++) {
    int i2 = i1 + 2;
    for (int iel = 1; iel <= nel; iel++) {
      int iel1 = C(ielel, i1, iel), iel2 = C(ielel, i2, iel);
      int j1 = C(ielfc, i1, iel), j2 = C(ielfc, i2, iel);
      double w1 = C(fcflux, j1, iel1), w2 = C(fcflux, j2, iel2);
      if (iel1 == iel) w1 = 0.0;
      if (iel2 == iel) w2 = 0.0;
      E(elflux, iel) = E(elflux, iel) - C(fcflux, i1, iel) - C(fcflux, i2, iel) + w1 + w2;
    }
  }
}

/* ale_kn_updateel (ale_kn_advectors.f90:155-180) */
static void ale_kn_updateel(int id1, int id2, int nel, const int *ielel, const int *ielfc,
                            const double *elbase0, const double *elbase1, const double *cut,
                            const double *fcflux, double *elflux, double *elvar) {
  ale_kn_sumflux(id1, id2, nel, ielel, ielfc, fcflux, elflux);
  for (int iel = 1; iel <= nel; iel++)
    if (E(elbase1, iel) > E(cut, iel))
      E(elvar, iel) = (E(elvar, iel) * E(elbase0, iel) + E(elflux, iel)) / E(elbase1, iel);
}

/* ale_kn_updatend (ale_kn_advectors.f90:182-214) */
static void ale_kn_updatend(int nnd, int nel, const int *ielnd, const double *ndbase0,
                            const double *ndbase1, const double *cut, const int *zactive,
                            const double *cnflux, double *ndflux, double *ndvar) {
  for (int ind = 1; ind <= nnd; ind++) E(ndflux, ind) = 0.0;
  for (int iel = 1; iel <= nel; iel++)
    for (int ii = 1; ii <= NCORN; ii++) {
      int ind = C(ielnd, ii, iel);
      E(ndflux, ind) = E(ndflux, ind) + C(cnflux, ii, iel);
    }
  for (int ind = 1; ind <= nnd; ind++)
    if (E(zactive, ind) && (E(ndbase1, ind) > E(cut, ind)))
      E(ndvar, ind) = (E(ndvar, ind) * E(ndbase0, ind) + E(ndflux, ind)) / E(ndbase1, ind);
}

/* ale_dr_advectel (ale_dr_advect.f90:102-127, 162-224) */
static void ale_dr_advectel(orc_ctx *ctx, int id1, int id2) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  /* ale_dr_advectbasisel */
  ale_kn_sumflux(id1, id2, s->nel, I(BL_IELEL), I(BL_IELFC), R(AL_FCDV), R(AL_RWORK1));
  ale_kn_fluxelvl(id1, id2, s->nel1, I(BL_IELEL), I(BL_IELFC), R(BL_CNWT), R(AL_FCDV),
                  R(BL_ELDENSITY), R(AL_FCDM));
  ale_kn_sumflux(id1, id2, s->nel, I(BL_IELEL), I(BL_IELFC), R(AL_FCDM), R(AL_RWORK2));
  ale_kn_updatebasisel(s->nel, c->zerocut, c->dencut, R(AL_RWORK1), R(AL_RWORK2), R(AL_STORE5),
                       R(AL_STORE6), R(AL_STORE1), R(AL_STORE2), R(AL_STORE3), R(BL_ELVOLUME),
                       R(BL_ELMASS), R(BL_ELDENSITY));
  /* ale_dr_advectvarel */
  ale_kn_fluxelvl(id1, id2, s->nel1, I(BL_IELEL), I(BL_IELFC), R(BL_CNMASS), R(AL_FCDM),
                  R(BL_ELENERGY), R(AL_FLUX));
  ale_kn_updateel(id1, id2, s->nel, I(BL_IELEL), I(BL_IELFC), R(AL_STORE2), R(BL_ELMASS),
                  R(AL_STORE6), R(AL_FLUX), R(AL_RWORK1), R(BL_ELENERGY));
}

/* ale_dr_advectnd (ale_dr_advect.f90:129-160, 226-305) */
static void ale_dr_advectnd(orc_ctx *ctx, int id1, int id2) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  utils_kn_cngather(s->nel, I(BL_IELND), R(BL_NDU), R(AL_CNU));
  utils_kn_cngather(s->nel, I(BL_IELND), R(BL_NDV), R(AL_CNV));
  /* ale_dr_advectbasisnd */
  ale_kn_initbasisnd(s->nnd2, R(AL_STORE3), R(AL_STORE4), R(AL_STORE2));
  ale_kn_calcbasisnd(s->nel2, I(BL_IELND), I(BL_IELSORT2), R(AL_STORE1), R(BL_ELVOLUME),
                     R(BL_CNMASS), R(AL_STORE3), R(AL_STORE4), R(AL_STORE2), R(AL_RWORK3));
  ale_kn_fluxbasisnd(id1, id2, s->nel2, I(BL_IELEL), I(BL_IELFC), I(BL_IELSORT2), R(AL_FCDV),
                     R(AL_FCDM), R(AL_RWORK1), R(AL_RWORK2), R(AL_FLUX));
  utils_kn_copy(s->nnd2, R(AL_STORE2), R(AL_STORE1));
  ale_kn_massbasisnd(s->nel2, I(BL_IELND), I(BL_IELSORT2), R(AL_FLUX), R(BL_CNMASS),
                     R(AL_STORE1));
  ale_kn_cutbasisnd(s->nnd, c->zerocut, c->dencut, R(AL_STORE3), R(AL_STORE5), R(AL_STORE6));
  /* ale_dr_advectvarnd */
  ale_kn_activend(s->nnd, -1, I(AL_INDSTATUS), I(BL_INDTYPE), I(AL_ZACTIVE));
  ale_kn_fluxndvl(s->nel1, I(BL_IELEL), I(BL_IELFC), R(AL_RWORK3), R(AL_RWORK2), R(AL_CNU),
                  R(AL_FLUX));
  ale_kn_updatend(s->nnd, s->nel1, I(BL_IELND), R(AL_STORE2), R(AL_STORE1), R(AL_STORE6),
                  I(AL_ZACTIVE), R(AL_FLUX), R(AL_FCDM), R(BL_NDU));
  ale_kn_activend(s->nnd, -2, I(AL_INDSTATUS), I(BL_INDTYPE), I(AL_ZACTIVE));
  ale_kn_fluxndvl(s->nel1, I(BL_IELEL), I(BL_IELFC), R(AL_RWORK3), R(AL_RWORK2), R(AL_CNV),
                  R(AL_FLUX));
  ale_kn_updatend(s->nnd, s->nel1, I(BL_IELND), R(AL_STORE2), R(AL_STORE1), R(AL_STORE6),
                  I(AL_ZACTIVE), R(AL_FLUX), R(AL_FCDM), R(BL_NDV));
}

/* ========================= solver entry points =========================== */

/* inf_solver_getdt (inf_solver_getdt.f90:35-70) with time_dr_calc and
 * time_dr_end (time_dr_advance.f90:38-132) */
int orc_getdt(orc_ctx *ctx, bl_timestep *ts, bl_error *error) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  dt_cand list[5];
  int n = 0;
  set_err(error, BL_SUCCESS, BL_HALT_SINGLE, "");
  /* time_dr_calc */
  list[n].rdt = c->dt_max; list[n].idt = -1; list[n].code = BL_DT_MAXIMUM; n++;
  list[n].rdt = c->dt_g * ts->dt; list[n].idt = -1; list[n].code = BL_DT_GROWTH; n++;
  if (ts->nstep == 0) { list[n].rdt = c->dt_initial; list[n].idt = -1; list[n].code = BL_DT_INITIAL; n++; }
  /* hydro_dr_getdt (hydro_dr_getdt.f90:39-79) */
  utils_kn_cngather(s->nel, I(BL_IELND), R(BL_NDU), R(DT_CNU));
  utils_kn_cngather(s->nel, I(BL_IELND), R(BL_NDV), R(DT_CNV));
  hydro_dr_getviscosity(ctx);
  hydro_dr_getcs2(ctx);
  if (hydro_kn_getdtcfl(ctx, &list[n]) != BL_SUCCESS) {
    set_err(error, BL_FAILURE, BL_HALT_SINGLE, "ERROR: negative CFL condition in hydro_dr_getdt");
    return BL_FAILURE;
  }
  n++;
  hydro_kn_getdtdiv(ctx, &list[n]);
  n++;
  /* ale_dr_getdt would run here only if ale%zon, which no input can set. */
  /* time_dr_end: smallest candidate, first one kept on ties */
  dt_cand mindt = list[0];
  for (int i = 1; i < n; i++)
    if (list[i].rdt < mindt.rdt) mindt = list[i];
  ts->nstep = ts->nstep + 1;
  ts->dt = mindt.rdt;
  time_set_sdt(ts, mindt.code);
  ts->idtel = mindt.idt;
  time_set_mdt(ctx, ts);
  ts->time = ts->time + ts->dt;
  if (ts->dt < c->dt_min) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: dt < dt_min");
    return BL_FAILURE;
  }
  return BL_SUCCESS;
}

/* inf_solver_getstate (inf_solver_lagstep.f90:80-103) */
static int inf_solver_getstate(orc_ctx *ctx, const bl_timestep *ts, bl_error *error) {
  const bl_sizes *s = &ctx->s;
  /* hydro_dr_getstate (hydro_dr_getstate.f90:33-51) */
  geometry_kn_getvertex(s->nnd, 0.5 * ts->dt, R(BL_NDX), R(BL_NDY), R(BL_NDU), R(BL_NDV));
  int ierr = geometry_dr_getgeometry(ctx);
  if (ierr != BL_SUCCESS) {
    set_err(error, ierr, BL_HALT_SINGLE, "ERROR: negative volume in geometry_dr_getgeometry");
    return ierr;
  }
  density_dr_getdensity(ctx);
  hydro_dr_getenergy(ctx, ts);
  eos_dr_geteos(ctx);
  return BL_SUCCESS;
}

/* inf_solver_lagstep (inf_solver_lagstep.f90:44-78) */
int orc_lagstep(orc_ctx *ctx, bl_timestep *ts, bl_error *error) {
  const bl_sizes *s = &ctx->s;
  set_err(error, BL_SUCCESS, BL_HALT_SINGLE, "");
  /* inf_solver_setpredictor: time_dr_setpredictor + hydro_dr_setpredictor */
  ts->zcorrector = 0;
  ts->dts = 0.5 * ts->dt;
  utils_kn_copy(s->nel, R(BL_ELENERGY), R(LG_ELENERGY0));
  hydro_dr_getforce(ctx, ts);
  int ierr = inf_solver_getstate(ctx, ts, error);
  if (ierr != BL_SUCCESS) return ierr;
  /* inf_solver_setcorrector */
  ts->zcorrector = 1;
  ts->dts = ts->dt;
  utils_kn_copy(s->nel, R(LG_ELENERGY0), R(BL_ELENERGY));
  hydro_dr_getforce(ctx, ts);
  inf_solver_getacceleration(ctx, ts);
  return inf_solver_getstate(ctx, ts, error);
}

/* inf_solver_alestep (inf_solver_alestep.f90:39-74) */
int orc_alestep(orc_ctx *ctx, const bl_timestep *ts, bl_error *error) {
  const bl_sizes *s = &ctx->s;
  const bl_config *c = &ctx->c;
  set_err(error, BL_SUCCESS, BL_HALT_SINGLE, "");
  /* ale_active (ale_dr_utils.f90:35-51) */
  if (!c->ale_zexist) return BL_SUCCESS;
  if (!((ts->time >= c->ale_mintime) && (ts->time <= c->ale_maxtime))) return BL_SUCCESS;
  /* ale_dr_getmeshstatus / ale_kn_getmeshstatus (ale_kn_getmeshstatus.f90:28-45) */
  if (c->ale_zeul)
    for (int ind = 1; ind <= s->nnd; ind++) E(I(AL_INDSTATUS), ind) = 2;
  /* ale_dr_getfluxvolume (ale_dr_getfluxvolume.f90:37-71) */
  if (c->ale_zeul) {
    /* ale_kn_getmeshvelocity (ale_kn_getmeshvelocity.f90:28-46) */
    for (int ind = 1; ind <= s->nnd; ind++) {
      E(R(AL_STORE4), ind) = -E(R(AL_STORE4), ind);
      E(R(AL_STORE5), ind) = -E(R(AL_STORE5), ind);
    }
  }
  utils_kn_copy(s->nnd, R(BL_NDX), R(AL_STORE2));
  utils_kn_copy(s->nnd, R(BL_NDY), R(AL_STORE3));
  geometry_kn_getvertex(s->nnd, ts->dt, R(BL_NDX), R(BL_NDY), R(AL_STORE4), R(AL_STORE5));
  geometry_kn_getfluxvolume(s->nel, c->zerocut, I(BL_IELND), R(AL_STORE2), R(AL_STORE3),
                            R(BL_NDX), R(BL_NDY), R(AL_FCDV));
  /* ale_dr_advect (ale_dr_advect.f90:56-100) */
  switch (c->ale_adv_type) {
    case 1:
      ale_dr_advectel(ctx, 1, 2);
      ale_dr_advectnd(ctx, 1, 2);
      break;
    case 2: {
      int ii = modF(ts->nstep + 1, 2);
      int i1 = 1 + ii, i2 = 2 - ii, i3 = i2 - i1;
      for (int d = i1;; d += i3) {
        ale_dr_advectel(ctx, d, d);
        ale_dr_advectnd(ctx, d, d);
        if (d == i2) break;
      }
      break;
    }
    default:
      set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: unrecognised adv_type");
      return BL_FAILURE;
  }
  /* inf_solver_aleupdate -> ale_dr_hydroupdate (ale_dr_update.f90:33-51) */
  int ierr = geometry_dr_getgeometry(ctx);
  density_dr_getdensity(ctx);
  eos_dr_geteos(ctx);
  if (ierr != BL_SUCCESS) {
    set_err(error, ierr, BL_HALT_SINGLE, "ERROR: negative volume in geometry_dr_getgeometry");
    return ierr;
  }
  return BL_SUCCESS;
}

/* ========================= lifetime ====================================== */

static long field_len(const bl_sizes *s, int id) {
  long nsz = s->nsz > 0 ? s->nsz : (s->nel > s->nnd ? s->nel : s->nnd);
  long mcp = s->mcp > s->ncp ? s->mcp : s->ncp;
  if (mcp < 1) mcp = 1;
  switch (id) {
    case BL_RSCRATCH21: case BL_RSCRATCH22: case BL_RSCRATCH23: case BL_RSCRATCH24:
    case BL_RSCRATCH25: case BL_RSCRATCH26: case BL_RSCRATCH27: case BL_RSCRATCH28:
      return 4 * nsz;
    case BL_RSCRATCH11: case BL_RSCRATCH12: case BL_RSCRATCH13: case BL_RSCRATCH14:
    case BL_RSCRATCH15: case BL_RSCRATCH16: case BL_RSCRATCH17: case BL_ISCRATCH11:
    case BL_ZSCRATCH11:
      return nsz;
    case BL_RCPSCRATCH21: case BL_RCPSCRATCH22: case BL_RCPSCRATCH23: case BL_RCPSCRATCH24:
      return 4 * mcp;
    case BL_RCPSCRATCH11: case BL_ICPSCRATCH11: case BL_ICPSCRATCH12:
      return mcp;
    default:
      return -1;
  }
}

orc_ctx *orc_init(const bl_sizes *sizes, const bl_config *config, void *const *dh,
                  bl_error *error) {
  orc_ctx *ctx = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  ctx->s = *sizes;
  ctx->c = *config;
  if (ctx->s.nsz <= 0) ctx->s.nsz = ctx->s.nel > ctx->s.nnd ? ctx->s.nel : ctx->s.nnd;
  for (int id = 1; id <= BL_NID; id++) {
    ctx->f[id] = dh ? dh[id] : NULL;
    long n = field_len(&ctx->s, id);
    if (!ctx->f[id] && n > 0) {
      ctx->f[id] = calloc((size_t)n, 8);
      ctx->own[id] = 1;
    }
  }
  set_err(error, BL_SUCCESS, BL_HALT_SINGLE, "");
  return ctx;
}

void orc_finalize(orc_ctx *ctx) {
  if (!ctx) return;
  for (int id = 1; id <= BL_NID; id++)
    if (ctx->own[id]) free(ctx->f[id]);
  free(ctx);
}

void *orc_field(orc_ctx *ctx, int id) { return (id >= 1 && id <= BL_NID) ? ctx->f[id] : NULL; }

/* ========================= Sod known-answer test ========================= */

/* sod (check_kn_tests.f90:64-111): exact Riemann solution for the reference
 * deck geometry (x in [0,100], interface at 50, gamma 1.4). */
static void sod_exact(double xx, double time, double res[2]) {
  res[0] = -DBL_MAX;
  res[1] = -DBL_MAX;
  double coeff = sqrt(1.4);
  if (xx <= -coeff * time) {
    res[0] = 1.0;
    res[1] = 2.5;
  } else if (xx <= -0.07027281256118326961 * time) {
    double ss = xx / time;
    double velocity = (5.0 / 6.0) * (ss + coeff);
    double tt = ((velocity - ss) * (velocity - ss)) / 1.4;
    res[0] = pow(tt, 2.5);
    res[1] = res[0] * tt / (0.4 * res[0]);
  } else if (xx <= 0.92745262004894994908 * time) {
    res[0] = 0.42631942817849519385;
    res[1] = 1.77760006942335264781;
  } else {
    if (time <= 28.53627624872492075028) {
      if (xx <= 1.75215573203017816370 * time) {
        res[0] = 0.26557371170530706471;
        res[1] = 2.85354088799095973738;
      } else {
        res[0] = 0.125;
        res[1] = 2.0;
      }
    } else if (time < 40.68191725689148697880) {
      if (xx <= (50.0 - (time - 28.53627624872492075028) * 1.01019363599101820444)) {
        res[0] = 0.26557371170530706471;
        res[1] = 2.85354088799095973738;
      } else {
        res[0] = 0.50939531774381657731;
        res[1] = 3.82996297061558546292;
      }
    }
  }
}

void orc_sod_l1(int nel, double time, const double *volume, const double *density,
                const double *energy, const double *cnx, const double *cny, double out[2]) {
  double basis = 0.0, l1[2] = {0.0, 0.0};
  for (int ii = 1; ii <= nel; ii++) {
    double c[2], sol[2];
    orc_centroid(4, &C(cnx, 1, ii), &C(cny, 1, ii), c);
    sod_exact(c[0] - 50.0, time, sol);
    basis = basis + E(volume, ii);
    l1[0] = fabs(E(density, ii) - sol[0]) * E(volume, ii) + l1[0];
    l1[1] = fabs(E(energy, ii) - sol[1]) * E(volume, ii) + l1[1];
  }
  out[0] = l1[0] / basis;
  out[1] = l1[1] / basis;
}
