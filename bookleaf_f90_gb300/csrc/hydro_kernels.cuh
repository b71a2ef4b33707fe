// hydro_kernels.cu -- the Lagrangian hot path on sm_103a.
//
// Four kernels per step replace the reference's sequence of loops:
//   k_getdt        inf_solver_getdt: utils_kn_cngather u,v; the three edge-
//                  viscosity loops (hydro_kn_edgeviscosity.f90:30-282);
//                  hydro_dr_getcs2; hydro_kn_getdtcfl / getdtdiv
//                  (hydro_kn_getdt.f90:30-122) with the two argmin/argmax
//                  scans done as a block reduction plus a last-block pass
//                  that also runs time_dr_end (time_dr_advance.f90:74-132).
//   k_lag_force    inf_solver_lagstep up to the corrector force: predictor
//                  force (hydro_kn_getforce.f90), half-step vertices,
//                  geometry, density, energy, EoS, then the corrector force
//                  with hourglass and sub-zonal terms, and the mixed-cell
//                  force average (hydro_dr_getacceleration.f90:61-79).
//   k_lag_accel    hydro_kn_scatteracceleration/getacceleration/
//                  applyacceleration and utils_kn_bc per node, gathering
//                  corner contributions over a CSR in the reference's loop
//                  order; writes u^{n+1}, ubar and the final vertices.
//   k_lag_state    the corrector getstate: geometry at x^{n+1}, density,
//                  energy from e^n with the corrector forces and ubar, EoS.
//
// Every expression keeps the reference's operand order.  This file is
// compiled twice: with --fmad=false (namespace exact) the results equal the
// CPU restatement bit for bit; with --fmad=true (namespace fast) the compiler
// may fuse multiply-adds.
#pragma once
#include <cfloat>
#include <cmath>

#include "bl_device.cuh"
#include "bl_elem.cuh"
#include "bl_fp64.cuh"
#include "bl_lreal.cuh"
#include "bl_kernels.h"
#include "bl_mma.cuh"

// Every FP64 division and square root of the per-element work goes
// through the integer-pipe versions, which return the IEEE results bit for
// bit (bl_fp64.cuh); the three of the dt reduction's last block, one
// thread on the kernel's serial tail, use the hardware's (the same bits at
// a fraction of the latency).
// The divides and square roots run out of line: one body per kernel instead
// of ~60 inlined copies of ~100 instructions, which overflowed the
// instruction cache (k_getdt stalled on instruction fetch); measured on the
// GB300 over the whole Sedov 512x512 run: 556.1M zone-cycles/s against
// 514.6M inlined.
#ifndef BL_DIV_CALL
#define BL_DIV_CALL 1
#endif
#if BL_DIV_CALL
namespace bl {
static __device__ __noinline__ double ddiv_call(double a, double b) { return ddiv_rn(a, b); }
static __device__ __noinline__ double dsqrt_call(double x) { return dsqrt_rn(x); }
}  // namespace bl
#define DIV(a, b) ::bl::ddiv_call((a), (b))
#define SQRT(a) ::bl::dsqrt_call(a)
#endif
#ifndef DIV
#define DIV(a, b) ::bl::ddiv_rn((a), (b))
#endif
#ifndef SQRT
#define SQRT(a) ::bl::dsqrt_rn(a)
#endif

// Resident blocks of 128 threads per SM the two heaviest kernels are
// compiled for (register budget 65536 / (128 * n) per thread).  Chosen by
// timing the whole Sedov 512x512 run on the GB300 over k_getdt n = 5..8
// and k_lag_force n = 2..6: 832.0M zone-cycles/s at 7 and 4 against 814.9M
// at 5 and 3, 822.0M at 7 and 3, 823.4M at 5 and 4.  k_getdt gains from
// the warps that hide its integer-pipe divide chains and from the 8,192
// warps of a 512x512 mesh filling 1.92 waves of 28 warps per SM instead of
// 2.69 waves of 20 (the last, part-filled wave drains at low occupancy).
#ifndef BL_GETDT_MINB
#define BL_GETDT_MINB 7
#endif
// The fast build's k_getdt as two kernels (BL_GETDT_SPLIT): the edge
// viscosity, then the dt scans and reduction.  Measured on Sedov 512x512:
// the same step time in FP64 (293.6-294.0 against 293.6-293.8 us), 4-5 %
// faster in the demoted form (k_getdt 62.1 against 68.7-71.0 us; 205.1
// against 215.0 us per step), which is latency-bound and whose halves run
// without spills; the build enables it for the demoted form only.
#ifndef BL_GETDT_SPLIT
#define BL_GETDT_SPLIT 0
#endif
// The fast build may also use exact algebraic identities that can change
// only the sign of a zero (negation symmetry of opposite corners); the
// exact build evaluates every expression as written.
#ifndef BL_FAST_ALGEBRA
#define BL_FAST_ALGEBRA 0
#endif
#ifndef BL_FORCE_MINB
#define BL_FORCE_MINB 4
#endif
// Minimum resident blocks per SM of the two short kernels (0: the plain
// block-size bound).  From the same whole-run sweep: k_lag_accel with a
// one-block bound takes 56 registers and no spills (24.8 us against 26.3 us
// at the 40 registers of the plain bound, 913.7M against 907.8M
// zone-cycles/s); k_lag_state is best with the plain bound (72 registers;
// 1, 8, 12 and 16 blocks were slower or equal).
#ifndef BL_ACCEL_MINB
#define BL_ACCEL_MINB 1
#endif
#ifndef BL_STATE_MINB
#define BL_STATE_MINB 0
#endif
#if BL_ACCEL_MINB > 0
#define BL_ACCEL_BOUNDS(bs) __launch_bounds__(bs, BL_ACCEL_MINB)
#else
#define BL_ACCEL_BOUNDS(bs) __launch_bounds__(bs)
#endif
#if BL_STATE_MINB > 0
#define BL_STATE_BOUNDS(bs) __launch_bounds__(bs, BL_STATE_MINB)
#else
#define BL_STATE_BOUNDS(bs) __launch_bounds__(bs)
#endif

namespace bl {
namespace BL_NS {

// ------------------------------------------------------------------ EoS
// eos_kn_getpressure / eos_kn_getcs2 (eos_kn_forms.f90:28-106)
__device__ __forceinline__ void eos_pc(const DevCfg& C, int mat, double rho, double e,
                                       double& p, double& cs2) {
  const int imat = mat > 0 ? mat : 0;
  const int t = __ldg(C.eos_type + imat);
  const double* P = C.eos_param + 6 * imat;
  if (t == 1) {
    p = e * rho * __ldg(C.eos_gm1 + imat);
    cs2 = __ldg(C.eos_ggm1 + imat) * e;
  } else if (t == 0) {
    p = __ldg(P);
    cs2 = C.ccut;
  } else if (t == 2) {
    double t1 = DIV(rho, __ldg(P + 2));
    p = __ldg(P) * (bl_pow(t1, __ldg(P + 1)) - 1.0);
    p = maxF(p, __ldg(P + 3));
    double t2 = __ldg(P + 1) - 1.0;
    cs2 = DIV(__ldg(P) * __ldg(P + 1), __ldg(P + 2));
    cs2 = cs2 * bl_pow(t1, t2);
  } else if (t == 3) {
    double t1 = DIV(__ldg(P + 3) * __ldg(P + 5), rho);
    double t2 = DIV(__ldg(P + 4) * __ldg(P + 5), rho);
    double t3 = __ldg(P) * rho * e;
    double t4 = (1.0 - DIV(__ldg(P), t1)) * __ldg(P + 1) * bl_exp(-t1);
    double t5 = (1.0 - DIV(__ldg(P), t2)) * __ldg(P + 2) * bl_exp(-t2);
    p = t3 + t4 + t5;
    double pp = p;
    if (gt_nn(C.pcut, absF(pp))) pp = 0.0;
    double q1 = DIV(__ldg(P + 5), rho);
    double s3 = __ldg(P + 3) * q1;
    double u4 = DIV(__ldg(P), __ldg(P + 3)) + __ldg(P) * q1 - s3 * q1;
    u4 = u4 * __ldg(P + 1) * bl_exp(-s3);
    s3 = __ldg(P + 4) * q1;
    double u5 = DIV(__ldg(P), __ldg(P + 4)) + __ldg(P) * q1 - s3 * q1;
    u5 = u5 * __ldg(P + 2) * bl_exp(-s3);
    cs2 = DIV(__ldg(P) * pp, rho) + __ldg(P) * e - u4 - u5;
  } else {
    p = -1.0;
    cs2 = C.ccut;
  }
  if (gt_nn(C.pcut, absF(p))) p = 0.0;
  cs2 = maxF(cs2, C.ccut);
}

// ------------------------------------------------------------------ geometry
// geometry_kn_getiso + getvolume (geometry_kn_volume.f90:30-79)
struct Iso {
  double a1, a2, a3, b1, b2, b3, w0, w1, w2, w3, vol;
  // fast build: a1*b3 - a3*b1 and the two skew products' sum and
  // difference, T1 + T3 and T3 - T1 with T1 = a1*b2 - a2*b1 and
  // T3 = a3*b2 - a2*b3 (shared with the sub-zonal pressure force)
  double cross, ts, td;
};

#if BL_FAST_ALGEBRA
// Fast build: the same quantities with fewer roundings.  a1 and a3 share
// the diagonal differences (x2-x0) +- (x1-x3).  Expanding the reference's
// corner weights, (3b3 -+ b2)(3a1 -+ a2) - (3a3 -+ a2)(3b1 -+ b2) over 9,
// gives cross + (T3 - T1)/3, cross + (T1 + T3)/3, cross - (T3 - T1)/3,
// cross - (T1 + T3)/3 for corners 0..3 (exact in real arithmetic).
__device__ __forceinline__ Iso getiso(const double* x, const double* y) {
  Iso g;
  const double ux = x[2] - x[0], vx = x[1] - x[3];
  const double uy = y[2] - y[0], vy = y[1] - y[3];
  g.a1 = quarter(ux + vx);
  g.a3 = quarter(ux - vx);
  g.a2 = quarter((x[0] + x[2]) - (x[1] + x[3]));
  g.b1 = quarter(uy + vy);
  g.b3 = quarter(uy - vy);
  g.b2 = quarter((y[0] + y[2]) - (y[1] + y[3]));
  g.cross = g.a1 * g.b3 - g.a3 * g.b1;
  const double t1 = g.a1 * g.b2 - g.a2 * g.b1;
  const double t3 = g.a3 * g.b2 - g.a2 * g.b3;
  g.ts = t1 + t3;
  g.td = t3 - t1;
  const double o3 = 1.0 / 3.0;
  g.w0 = fma(g.td, o3, g.cross);
  g.w1 = fma(g.ts, o3, g.cross);
  g.w2 = fma(-g.td, o3, g.cross);
  g.w3 = fma(-g.ts, o3, g.cross);
  g.vol = times4(g.cross);
  return g;
}
#else
__device__ __forceinline__ Iso getiso(const double* x, const double* y) {
  Iso g;
  g.a1 = quarter(-x[0] + x[1] + x[2] - x[3]);
  g.a2 = quarter(x[0] - x[1] + x[2] - x[3]);
  g.a3 = quarter(-x[0] - x[1] + x[2] + x[3]);
  g.b1 = quarter(-y[0] + y[1] + y[2] - y[3]);
  g.b2 = quarter(y[0] - y[1] + y[2] - y[3]);
  g.b3 = quarter(-y[0] - y[1] + y[2] + y[3]);
  const double o9 = 1.0 / 9.0;
  const double A1m = 3.0 * g.a1 - g.a2, A1p = 3.0 * g.a1 + g.a2;
  const double A3m = 3.0 * g.a3 - g.a2, A3p = 3.0 * g.a3 + g.a2;
  const double B1m = 3.0 * g.b1 - g.b2, B1p = 3.0 * g.b1 + g.b2;
  const double B3m = 3.0 * g.b3 - g.b2, B3p = 3.0 * g.b3 + g.b2;
  g.w0 = o9 * (B3m * A1m - A3m * B1m);
  g.w1 = o9 * (B3p * A1m - A3p * B1m);
  g.w2 = o9 * (B3p * A1p - A3p * B1p);
  g.w3 = o9 * (B3m * A1p - A3m * B1p);
  g.vol = times4(g.a1 * g.b3 - g.a3 * g.b1);
  g.cross = g.ts = g.td = 0.0;
  return g;
}
#endif

// geometry_kn_length (geometry_kn_length.f90:99-139)
__device__ __forceinline__ double g_denom(double x1, double y1, double x2, double y2) {
  double w1 = y1 - y2, w2 = x1 - x2;
  return w1 * w1 + w2 * w2;
}
__device__ __forceinline__ double g_distpp(double x3, double y3, double x4, double y4, double x1,
                                           double y1) {
  double w1 = half(x3 + x4) - x1;
  double w2 = half(y3 + y4) - y1;
  return w1 * w1 + w2 * w2;
}
__device__ __forceinline__ double g_distpl(double x3, double y3, double x4, double y4, double x1,
                                           double y1, double x2, double y2) {
  double res = half(y1 - y2) * (x3 + x4) + half(y3 + y4) * (x2 - x1) + y2 * x1 - y1 * x2;
  return res * res;
}

// MINVAL(geometry_kn_dln(...)) (geometry_kn_length.f90:58-97)
__device__ __forceinline__ double min_dln(const double* x, const double* y, double zcut) {
  double r[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    // res(k+1): denominator from corners k+2,k+3; distance of corners
    // k,k+1 midpoint... in the reference's argument order
    const int a = k, b = (k + 1) & 3, c = (k + 2) & 3, d = (k + 3) & 3;
    double w1 = g_denom(x[c], y[c], x[d], y[d]);
    if (gt_nn(zcut, w1)) r[k] = g_distpp(x[a], y[a], x[b], y[b], x[c], y[c]);
    else r[k] = DIV(g_distpl(x[a], y[a], x[b], y[b], x[c], y[c], x[d], y[d]), w1);
  }
  double m = r[0];  // all four are sums of squares or their quotients
  m = minF_nn(m, r[1]);
  m = minF_nn(m, r[2]);
  m = minF_nn(m, r[3]);
  return m;
}

#if BL_FAST_ALGEBRA
// Fast build: the same squared lengths from the element's iso-parametric
// coefficients.  For side k the opposite edge (corners k+2 -> k+3) is
// 2*(dx,dy) with (dx,dy) = (a1+a2, b1+b2), (a2-a3, b2-b3), (a1-a2, b1-b2),
// (a2+a3, b2+b3), and its cross product with the vector to the midpoint of
// corners k,k+1 is 4*(dx*q - dy*p) with (p,q) = (a3,b3), (a1,b1), (a3,b3),
// (a1,b1); so the reference's distpl/denom is 4 X^2 / Y with X = dx*q -
// dy*p and Y = dx^2 + dy^2 (exact in real arithmetic), and its denominator
// is 4 Y.  A degenerate opposite edge (4 Y < zcut) takes the corner form.
// (T: FP64, or FP32 in the mixed build)
template <class T>
__device__ __forceinline__ T min_dln_iso(const double* x, const double* y, T zcut, T a1, T a2,
                                         T a3, T b1, T b2, T b3) {
  const T dxs[4] = {a1 + a2, a2 - a3, a1 - a2, a2 + a3};
  const T dys[4] = {b1 + b2, b2 - b3, b1 - b2, b2 + b3};
  T r[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const T dx = dxs[k], dy = dys[k];
    const T p = (k & 1) ? a1 : a3, q = (k & 1) ? b1 : b3;
    const T Y = dx * dx + dy * dy;
    if (gt_nn(zcut, times4(Y))) {
      const int a = k, b = (k + 1) & 3, c = (k + 2) & 3;
      r[k] = (T)g_distpp(x[a], y[a], x[b], y[b], x[c], y[c]);
    } else {
      const T X = dx * q - dy * p;
      r[k] = DIV(times4(X * X), Y);
    }
  }
  T m = r[0];
  m = minF_nn(m, r[1]);
  m = minF_nn(m, r[2]);
  m = minF_nn(m, r[3]);
  return m;
}
#endif

// MINVAL(geometry_kn_dlm(...)) (geometry_kn_length.f90:30-56)
__device__ __forceinline__ double min_dlm(const double* x, const double* y) {
  double x1 = x[0] + x[1], x2 = x[2] + x[3], y1 = y[0] + y[1], y2 = y[2] + y[3];
  x1 = half(x1 - x2);
  y1 = half(y1 - y2);
  double r0 = x1 * x1 + y1 * y1;
  x1 = x[2] + x[1];
  x2 = x[0] + x[3];
  y1 = y[2] + y[1];
  y2 = y[0] + y[3];
  x1 = half(x1 - x2);
  y1 = half(y1 - y2);
  double r1 = x1 * x1 + y1 * y1;
  double m = r0;
  m = minF_nn(m, r1);
  m = minF_nn(m, r0);
  m = minF_nn(m, r1);
  return m;
}

// ------------------------------------------------------------------ forces
// hydro_kn_getforceP + getforceQ (hydro_kn_getforce.f90:30-71)
__device__ __forceinline__ void force_pq(double p, double a1, double a3, double b1, double b3,
                                         const d4& qx, const d4& qy, double* fx,
                                         double* fy) {
#if BL_FAST_ALGEBRA
  // opposite corners carry opposite coefficients: b3 - b1 = -(b1 - b3)
  // exactly, up to the sign of a zero.  The four sums are the ones the
  // sub-zonal pressure force uses too.
  const double db = b1 - b3, sb = b1 + b3, da = a1 - a3, sa = a1 + a3;
  fx[0] = fma(p, db, qx.x);
  fx[1] = fma(p, sb, qx.y);
  fx[2] = fma(-p, db, qx.z);
  fx[3] = fma(-p, sb, qx.w);
  fy[0] = fma(-p, da, qy.x);
  fy[1] = fma(-p, sa, qy.y);
  fy[2] = fma(p, da, qy.z);
  fy[3] = fma(p, sa, qy.w);
#else
  fx[0] = p * (-b3 + b1);
  fx[1] = p * (b3 + b1);
  fx[2] = p * (b3 - b1);
  fx[3] = p * (-b3 - b1);
  fy[0] = p * (a3 - a1);
  fy[1] = p * (-a3 - a1);
  fy[2] = p * (-a3 + a1);
  fy[3] = p * (a3 + a1);
  fx[0] = fx[0] + qx.x;
  fy[0] = fy[0] + qy.x;
  fx[1] = fx[1] + qx.y;
  fy[1] = fy[1] + qy.y;
  fx[2] = fx[2] + qx.z;
  fy[2] = fy[2] + qy.z;
  fx[3] = fx[3] + qx.w;
  fy[3] = fy[3] + qy.w;
#endif
}

#if BL_FAST_ALGEBRA
// Fast build: hydro_kn_getforceSP (hydro_kn_getforce.f90:109-188) from the
// element's iso-parametric coefficients.  With the corners written as
// s - a1 + a2 - a3, s + a1 - a2 - a3, s + a1 + a2 + a3, s - a1 - a2 + a3
// (s the centroid), the sub-quad of corner j (the corner, the edge midpoint
// after it, the centroid, the edge midpoint before it) has the x
// coefficients (w3, w4) = (P, Q), (R, -P), (-S, -R), (-Q, S), all over 4,
// with P = 2a1 - a2, Q = 2a3 - a2, R = 2a3 + a2, S = 2a1 + a2, and the y
// coefficients (w5, w6) likewise from the b's.  Expanding (all exact in
// real arithmetic):
// - the sub-volumes 4(w3 w6 - w4 w5) are V_j = cross + td/2, cross + ts/2,
//   cross - td/2, cross - ts/2 (cross = a1 b3 - a3 b1, ts = T1 + T3,
//   td = T3 - T1, T1 = a1 b2 - a2 b1, T3 = a3 b2 - a2 b3);
// - with p_j = cs2 (spmass_j / V_j - rho), the reference's corner x forces
//   lfx(j,1) = p_j (w5 - w6) and lfx(j,2) = p_j (w5 + w6) are p_j c_j / 2
//   and p_j C_j / 2 with c = (db, sb, -db, -sb) and
//   C = (sb - b2, b2 - db, -(sb + b2), db + b2), db = b1 - b3, sb = b1 + b3;
//   lfx(j,3) and lfx(j,4) are their negatives;
// - in the reference's gather of the sub-quad forces to the corners the
//   midpoint terms of adjacent sub-quads cancel pairwise, leaving, with
//   M_j = p_j C_j and G = db (p0 - p2) + sb (p1 - p3),
//   fx0 += w1/8 (4 p0 db + 2 (M3 - M1) - G),
//   fx1 += w1/8 (4 p1 sb + 2 (M0 - M2) - G),
//   fx2 -= w1/8 (4 p2 db + 2 (M3 - M1) + G),
//   fx3 -= w1/8 (4 p3 sb + 2 (M0 - M2) + G);
// - the y forces are the same with the a's in place of the b's and the
//   sign of w1 reversed.
__device__ __forceinline__ void sp_direction(double k, const double* p, double e02, double e13,
                                             double c1, double c2, double c3, double* f) {
  const double dd = c1 - c3, ss = c1 + c3;
  const double m0 = p[0] * (ss - c2), m1 = p[1] * (c2 - dd);
  const double m2 = -(p[2] * (ss + c2)), m3 = p[3] * (dd + c2);
  const double d13 = twice(m3 - m1), d02 = twice(m0 - m2);
  const double g = fma(dd, e02, ss * e13);
  const double d4 = times4(dd), s4 = times4(ss);
  f[0] = fma(k, fma(p[0], d4, d13) - g, f[0]);
  f[1] = fma(k, fma(p[1], s4, d02) - g, f[1]);
  f[2] = fma(-k, fma(p[2], d4, d13) + g, f[2]);
  f[3] = fma(-k, fma(p[3], s4, d02) + g, f[3]);
}

__device__ __forceinline__ void force_sp_iso(double w1, double rho, double cs2, double cross,
                                             double ts, double td, double a1, double a2,
                                             double a3, double b1, double b2, double b3,
                                             const d4& spm, double* fx, double* fy) {
  const double V[4] = {fma(td, 0.5, cross), fma(ts, 0.5, cross), fma(-td, 0.5, cross),
                       fma(-ts, 0.5, cross)};
  const double cr = cs2 * rho;
  double p[4];
#pragma unroll
  for (int j = 0; j < 4; j++) p[j] = fma(cs2, DIV(c4(spm, j), V[j]), -cr);
  const double e02 = p[0] - p[2], e13 = p[1] - p[3];
  const double k = ldexpF<-3>(w1);
  sp_direction(k, p, e02, e13, b1, b2, b3, fx);
  sp_direction(-k, p, e02, e13, a1, a2, a3, fy);
}
#else
// hydro_kn_getforceSP (hydro_kn_getforce.f90:109-188)
__device__ void force_sp(double w1, double rho, double cs2, const double* cx, const double* cy,
                         const d4& spm, double* fx, double* fy) {
  double x3 = quarter(cx[0] + cx[1] + cx[2] + cx[3]);
  double y3 = quarter(cy[0] + cy[1] + cy[2] + cy[3]);
  // edge midpoints: x2 of corner j and x4 of corner j+1 are the same sum
  // (IEEE addition commutes), so each is evaluated once
  double mx[4], my[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    mx[j] = half(cx[j] + cx[(j + 1) & 3]);
    my[j] = half(cy[j] + cy[(j + 1) & 3]);
  }
  double lfx[4][4], lfy[4][4];
#pragma unroll
  for (int j1 = 0; j1 < 4; j1++) {
    double x1 = cx[j1], y1 = cy[j1];
    double x2 = mx[j1], y2 = my[j1];
    double x4 = mx[(j1 + 3) & 3], y4 = my[(j1 + 3) & 3];
    double w3 = quarter(-x1 + x2 + x3 - x4);
    double w4 = quarter(-x1 - x2 + x3 + x4);
    double w5 = quarter(-y1 + y2 + y3 - y4);
    double w6 = quarter(-y1 - y2 + y3 + y4);
    double w2 = times4(w3 * w6 - w4 * w5);
    w2 = DIV(c4(spm, j1), w2);
    w2 = w2 - rho;
    w2 = cs2 * w2;
    lfx[j1][0] = w2 * (w5 - w6);
    lfx[j1][1] = w2 * (w5 + w6);
    lfx[j1][2] = w2 * (-w5 + w6);
    lfx[j1][3] = w2 * (-w5 - w6);
    lfy[j1][0] = w2 * (-w3 + w4);
    lfy[j1][1] = w2 * (-w3 - w4);
    lfy[j1][2] = w2 * (w3 - w4);
    lfy[j1][3] = w2 * (w3 + w4);
  }
  double w2 = half(lfx[0][3] + lfx[3][1]);
  double w3 = half(lfx[0][1] + lfx[1][3]);
  double w4 = half(lfx[1][1] + lfx[2][3]);
  double w5 = half(lfx[3][3] + lfx[2][1]);
  double w6 = quarter(lfx[0][2] + lfx[1][2] + lfx[2][2] + lfx[3][2]);
  fx[0] = fx[0] + w1 * (lfx[0][0] + w2 + w3 + w6);
  fx[1] = fx[1] + w1 * (lfx[1][0] + w4 + w3 + w6);
  fx[2] = fx[2] + w1 * (lfx[2][0] + w4 + w5 + w6);
  fx[3] = fx[3] + w1 * (lfx[3][0] + w2 + w5 + w6);
  w2 = half(lfy[0][3] + lfy[3][1]);
  w3 = half(lfy[0][1] + lfy[1][3]);
  w4 = half(lfy[1][1] + lfy[2][3]);
  w5 = half(lfy[3][3] + lfy[2][1]);
  w6 = quarter(lfy[0][2] + lfy[1][2] + lfy[2][2] + lfy[3][2]);
  fy[0] = fy[0] + w1 * (lfy[0][0] + w2 + w3 + w6);
  fy[1] = fy[1] + w1 * (lfy[1][0] + w4 + w3 + w6);
  fy[2] = fy[2] + w1 * (lfy[2][0] + w4 + w5 + w6);
  fy[3] = fy[3] + w1 * (lfy[3][0] + w2 + w5 + w6);
}
#endif

// hydro_kn_getforceHG (hydro_kn_getforce.f90:73-107)
__device__ __forceinline__ void force_hg(double kappa, double rho, double area, double rdt,
                                         const double* u, const double* v, double* fx,
                                         double* fy) {
  double w2 = u[0] - u[1] + u[2] - u[3];
  double w3 = v[0] - v[1] + v[2] - v[3];
  double w1 = -kappa * rho * area * rdt;
  w2 = w1 * w2;
  w3 = w1 * w3;
  fx[0] = fx[0] + w2;
  fx[1] = fx[1] - w2;
  fx[2] = fx[2] + w2;
  fx[3] = fx[3] - w2;
  fy[0] = fy[0] + w3;
  fy[1] = fy[1] - w3;
  fy[2] = fy[2] + w3;
  fy[3] = fy[3] - w3;
}

// hydro_kn_getenergy (hydro_kn_getenergy.f90:29-52): the increment w1*dt
__device__ __forceinline__ double energy_update(double e, double m, double zerocut, double dt,
                                                const double* fx, const double* fy,
                                                const double* u, const double* v) {
  double w1 = fx[0] * u[0] + fy[0] * v[0] + fx[1] * u[1] + fy[1] * v[1] + fx[2] * u[2] +
              fy[2] * v[2] + fx[3] * u[3] + fy[3] * v[3];
  w1 = -DIV(w1, maxF(m, zerocut));
  return e + w1 * dt;
}

__device__ __forceinline__ bool halted(const DevStep* S) {
  return *((volatile const int*)&S->halted) != 0;
}

// The step header of an element's or a node's mesh: the context's single
// header, or in a batch the header of the mesh it belongs to; and the first
// element of that mesh (element numbers reported to the host are local to
// their mesh).
template <bool BATCH>
__device__ __forceinline__ DevStep* el_step(const DevFields& F, int iel) {
  return BATCH ? F.steps + __ldg(F.elinst + iel) : F.step;
}
template <bool BATCH>
__device__ __forceinline__ DevStep* nd_step(const DevFields& F, int ind) {
  return BATCH ? F.steps + __ldg(F.ndinst + ind) : F.step;
}
template <bool BATCH>
__device__ __forceinline__ int el_base(const DevFields& F, int iel) {
  return BATCH ? F.inst[__ldg(F.elinst + iel)].el_begin : 0;
}

// ================================================================ k_getdt

// (value,index) pairs for the two scans.  CFL: smallest value, first index
// on ties (hydro_kn_getdt.f90:70-73).  DIV: largest value above TINY, first
// index on ties, (TINY,-1) when no element exceeds TINY (:103-116).
__device__ __forceinline__ void cfl_min(double& v, int& i, double ov, int oi) {
  const long long ko = okey(ov), kv = okey(v);
  const bool ord = !nanF(ov) && !nanF(v);
  if (ord && (ko < kv || (ko == kv && oi < i))) { v = ov; i = oi; }
}
// DIV candidates are TINY or values that exceeded it: positive, never NaN,
// so their bit patterns order as integers
__device__ __forceinline__ void div_max(double& v, int& i, double ov, int oi) {
  const long long io = bits64(ov), iv = bits64(v);
  if (io > iv || (io == iv && oi >= 0 && (i < 0 || oi < i))) { v = ov; i = oi; }
}

// hydro_dr_getcs2 (elcs2 += elvisc; mixed cells: sum frmass*(cpcs2+cpvisc)),
// then the element's hydro_kn_getdtcfl and getdtdiv candidates
// How k_getdt reads an element's connectivity and region and stores its
// corner forces: in the library's own layout (0-based rows of four, face
// numbers packed in one int, 32-byte corner vectors).  The exact-form
// kernel takes the layout as a parameter, so that bl_getdt_noalloc runs the
// same kernel on arrays in the reference's layout.
struct DevLayout {
  static __device__ __forceinline__ int4 nodes(const DevFields& F, int e) {
    return __ldg(F.ielnd + e);
  }
  static __device__ __forceinline__ int4 nbrs(const DevFields& F, int e) {
    return __ldg(F.ielel + e);
  }
  static __device__ __forceinline__ int faces(const DevFields& F, int e) {
    return __ldg(F.ielfc + e);
  }
  static __device__ __forceinline__ int reg(const DevFields& F, int e) {
    return __ldg(F.ielreg + e);
  }
  static __device__ __forceinline__ void corners(d4* p, int e, const double* q) {
    p[e] = make_d4(q[0], q[1], q[2], q[3]);
  }
};

// The element's squared CFL length of hydro_kn_getdtcfl (min over its
// sides of geometry_kn_dlm or _dln), or -1 for a zdtnotreg region (the
// reference's HUGE candidate); it does not depend on the viscosity.
template <class L = DevLayout>
__device__ __forceinline__ double getdt_cfl_len(const DevFields& F, const DevCfg& C, int iel,
                                                const double* x, const double* y) {
  const int ireg = L::reg(F, iel);
  if (__ldg(C.zdtnotreg + ireg)) return -1.0;
#if BL_FAST_ALGEBRA
  return __ldg(C.zmidlength + ireg)
             ? min_dlm(x, y)
             : from_lr(min_dln_iso<lr>(x, y, lr_cut(C.zcut), to_lr(F.a1[iel]), to_lr(F.a2[iel]),
                                       to_lr(F.a3[iel]), to_lr(F.b1[iel]), to_lr(F.b2[iel]),
                                       to_lr(F.b3[iel])));
#else
  return __ldg(C.zmidlength + ireg) ? min_dlm(x, y) : min_dln(x, y, C.zcut);
#endif
}

// hydro_kn_getdtdiv's candidate of the element
__device__ __forceinline__ void getdt_div(const DevFields& F, int iel, const double* u,
                                          const double* v, double& divv, int& divi) {
#if BL_MIXED
  const lr A1 = to_lr(F.a1[iel]), A3 = to_lr(F.a3[iel]), B1 = to_lr(F.b1[iel]), B3 = to_lr(F.b3[iel]);
  lr wl = to_lr(u[0]) * (-B3 + B1) + to_lr(v[0]) * (A3 - A1) + to_lr(u[1]) * (B3 + B1) +
          to_lr(v[1]) * (-A3 - A1) + to_lr(u[2]) * (B3 - B1) + to_lr(v[2]) * (-A3 + A1) +
          to_lr(u[3]) * (-B3 - B1) + to_lr(v[3]) * (A3 + A1);
  const double w1 = from_lr(DIV(absF(wl), to_lr(F.vol[iel])));
#else
  const double A1 = F.a1[iel], A3 = F.a3[iel], B1 = F.b1[iel], B3 = F.b3[iel];
  double w1 = u[0] * (-B3 + B1) + v[0] * (A3 - A1) + u[1] * (B3 + B1) + v[1] * (-A3 - A1) +
              u[2] * (B3 - B1) + v[2] * (-A3 + A1) + u[3] * (-B3 - B1) + v[3] * (A3 + A1);
  w1 = DIV(absF(w1), F.vol[iel]);
#endif
  if (gt_nn(w1, divv)) {  // divv is TINY or a larger positive value
    divv = w1;
    divi = iel;
  }
}

// hydro_dr_getcs2 (elcs2 += elvisc; mixed cells: sum frmass*(cpcs2+cpvisc))
// and the element's CFL candidate from its squared length len
// (getdt_cfl_len)
__device__ __forceinline__ void getdt_cfl(const DevFields& F, int iel, double len, double visc,
                                          double& cflv, int& cfli) {
  double cs2v = F.cs2[iel] + visc;
  const int imx = F.elmx ? F.elmx[iel] : -1;
  if (imx >= 0) {
    double w1 = 0.0;
    const int c0 = F.imxfcp[imx], nc = F.imxncp[imx];
    for (int k = 0; k < nc; k++) w1 = w1 + F.frm[c0 + k] * (F.cpcs2[c0 + k] + F.cpvisc[c0 + k]);
    cs2v = w1;
  }
  F.cs2v[iel] = cs2v;
#if BL_MIXED
  const double r11 = len < 0.0 ? DBL_MAX : from_lr(DIV(to_lr(len), to_lr(cs2v)));
#else
  const double r11 = len < 0.0 ? DBL_MAX : DIV(len, cs2v);
#endif
  if (cfli == 0x7fffffff) {
    cflv = r11;
    cfli = iel;
  } else {
    cfl_min(cflv, cfli, r11, iel);
  }
}

// hydro_dr_getcs2, then the element's hydro_kn_getdtcfl and getdtdiv
// candidates
template <class L = DevLayout>
__device__ __forceinline__ void getdt_tail(const DevFields& F, const DevCfg& C, int iel,
                                           const double* x, const double* y, const double* u,
                                           const double* v, double visc, double& cflv, int& cfli,
                                           double& divv, int& divi) {
  getdt_cfl(F, iel, getdt_cfl_len<L>(F, C, iel, x, y), visc, cflv, cfli);
  getdt_div(F, iel, u, v, divv, divi);
}

// The block reduction of the candidates, the last block's reduction of the
// block partials and time_dr_end (time_dr_advance.f90:74-132)
// over the k_getdt blocks [blk0, blk0 + nblk) of one mesh (all of them for
// a single mesh; a batch's mesh in a batch, whose time-step parameters then
// come from I, and whose element numbers start at el0)
template <int BS, bool BATCH>
__device__ __forceinline__ void getdt_finish(const DevFields& F, const DevCfg& C, DevStep* S,
                                             double cflv, int cfli, double divv, int divi,
                                             int blk0, int nblk, int el0, const DevInst* I) {
  // ---- block reduction
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, cflv, o);
    int oi = __shfl_xor_sync(0xffffffffu, cfli, o);
    cfl_min(cflv, cfli, ov, oi);
    ov = __shfl_xor_sync(0xffffffffu, divv, o);
    oi = __shfl_xor_sync(0xffffffffu, divi, o);
    div_max(divv, divi, ov, oi);
  }
  __shared__ double s_cv[BS / 32], s_dv[BS / 32];
  __shared__ int s_ci[BS / 32], s_di[BS / 32];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    s_cv[wid] = cflv;
    s_ci[wid] = cfli;
    s_dv[wid] = divv;
    s_di[wid] = divi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < BS / 32; w++) {
      cfl_min(cflv, cfli, s_cv[w], s_ci[w]);
      div_max(divv, divi, s_dv[w], s_di[w]);
    }
    F.red_v[2 * blockIdx.x] = cflv;
    F.red_i[2 * blockIdx.x] = cfli;
    F.red_v[2 * blockIdx.x + 1] = divv;
    F.red_i[2 * blockIdx.x + 1] = divi;
    __threadfence();
    unsigned int t = atomicAdd(&S->ticket, 1u);
    s_last = (t == (unsigned int)(nblk - 1));
  }
  __syncthreads();
  if (!s_last) return;
  // ---- last block: reduce the partials, then time_dr_end
  __threadfence();
  cflv = HUGE_VAL;
  cfli = 0x7fffffff;
  divv = DBL_MIN;
  divi = -1;
  // Each thread takes the partials b = tid, tid + BS, ... in that order as
  // before, eight at a time: their loads (L2, past the L1 that may not see
  // other blocks' writes) are all in flight before the first comparison.
  // (Sixteen at a time, one round fewer on a 512x512 mesh, spilled in the
  // rest of the kernel and made it slower.)
  {
    constexpr int U = 8;
    const double2* rv = reinterpret_cast<const double2*>(F.red_v) + blk0;
    const int2* ri = reinterpret_cast<const int2*>(F.red_i) + blk0;
    const int nb = nblk;
    for (int b0 = threadIdx.x; b0 < nb; b0 += BS * U) {
      double2 v[U];
      int2 ix[U];
#pragma unroll
      for (int t = 0; t < U; t++) {
        const int b = b0 + t * BS;
        if (b < nb) {
          v[t] = __ldcg(rv + b);
          ix[t] = __ldcg(ri + b);
        }
      }
#pragma unroll
      for (int t = 0; t < U; t++) {
        if (b0 + t * BS < nb) {
          cfl_min(cflv, cfli, v[t].x, ix[t].x);
          div_max(divv, divi, v[t].y, ix[t].y);
        }
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, cflv, o);
    int oi = __shfl_xor_sync(0xffffffffu, cfli, o);
    cfl_min(cflv, cfli, ov, oi);
    ov = __shfl_xor_sync(0xffffffffu, divv, o);
    oi = __shfl_xor_sync(0xffffffffu, divi, o);
    div_max(divv, divi, ov, oi);
  }
  __syncthreads();
  if (lane == 0) {
    s_cv[wid] = cflv;
    s_ci[wid] = cfli;
    s_dv[wid] = divv;
    s_di[wid] = divi;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < BS / 32; w++) {
    cfl_min(cflv, cfli, s_cv[w], s_ci[w]);
    div_max(divv, divi, s_dv[w], s_di[w]);
  }
  S->ticket = 0;
  // time_dr_calc candidates then hydro's CFL and DIV (time_dr_advance.f90)
  if (cflv < 0.0) {  // hydro_kn_getdtcfl FAILURE
    S->ierr = -1;
    S->iout = 2;
    S->err_code = 1;
    if (S->run_mode) S->halted = 1;
    return;
  }
  // one thread's three operations: the hardware's correctly rounded
  // square root and divide (the same results as the integer-pipe routines,
  // at a fraction of their latency on the serial tail)
  const double rdt_cfl = C.cfl_sf * sqrt(cflv);
  const double rdt_div = C.div_sf / divv;
  // 1-based element numbers local to the mesh (0: none)
  const int cfln = cfli >= 0 && cfli != 0x7fffffff ? cfli - el0 + 1 : 0;
  const int divn = divi >= 0 ? divi - el0 + 1 : 0;
  const double dt_max = BATCH ? I->dt_max : C.dt_max, dt_g = BATCH ? I->dt_g : C.dt_g;
  const double dt_initial = BATCH ? I->dt_initial : C.dt_initial;
  const double dt_min = BATCH ? I->dt_min : C.dt_min, time_end = BATCH ? I->time_end : C.time_end;
  S->cfl_rdt = rdt_cfl;
  S->cfl_idt = cfln;
  S->div_rdt = rdt_div;
  S->div_idt = divn;
  double mind = dt_max;
  int mini = -1, mins = 0;
  double g = dt_g * S->dt;
  if (g < mind) { mind = g; mini = -1; mins = 1; }
  if (S->nstep == 0 && dt_initial < mind) { mind = dt_initial; mini = -1; mins = 2; }
  if (rdt_cfl < mind) { mind = rdt_cfl; mini = cfln; mins = 3; }
  if (rdt_div < mind) { mind = rdt_div; mini = divn; mins = 4; }
  S->nstep = S->nstep + 1;
  S->dt = mind;
  S->rdt = 1.0 / mind;
  S->sdt = mins;
  S->idtel = mini;
  S->time = S->time + mind;
  if (mind < dt_min) {
    S->ierr = -1;
    S->iout = 1;
    S->err_code = 2;
    if (S->run_mode) S->halted = 1;
  }
  if (S->run_mode) {
    if (S->time >= time_end) S->stop_next = 1;
    int r = S->nrecord;
    if (F.hist && r < C.max_records) {
      F.hist[r].time = S->time;
      F.hist[r].dt = S->dt;
      F.hist[r].nstep = S->nstep;
      F.hist[r].idtel = S->idtel;
      F.hist[r].sdt_code = S->sdt;
      F.hist[r].ierr = S->ierr;
    }
    S->nrecord = r + 1;
  }
}

#if BL_FAST_ALGEBRA
// Fast build.  The quantities of a face that both elements sharing it
// compute -- its lengths, unit vectors and the inverse ratio of its
// projections -- from the face's velocity (du, dv) and position (dx, dy)
// differences; the face vectors' projections on their own unit vectors
// are |d|^2 / max(|d|, zerocut) (exact in real arithmetic, never negative,
// so the reference's sign guards drop out).
// (in lr: FP64, or FP32 in the mixed build)
struct FaceQ {
  lr du, dv, lu, lx, uh, vh, xh, yh, w1;
};
__device__ __forceinline__ FaceQ face_q(lr du, lr dv, lr dx, lr dy, lr zc) {
  FaceQ f;
  f.du = du;
  f.dv = dv;
  const lr squ = du * du + dv * dv, sqx = dx * dx + dy * dy;
  f.lu = SQRT(squ);
  f.lx = SQRT(sqx);
  const lr ru = DIV((lr)1, maxF_nn(f.lu, zc)), rx = DIV((lr)1, maxF_nn(f.lx, zc));
  f.uh = du * ru;
  f.vh = dv * ru;
  f.xh = dx * rx;
  f.yh = dy * rx;
  const lr w1 = DIV(squ * ru, maxF_nn(sqx * rx, zc));
  f.w1 = DIV((lr)1, maxF_nn(w1, zc));
  return f;
}
// limiter ratio of a neighbour face with differences (ddx, ddy, ddu, ddv)
// against face f (hydro_kn_edgeviscosity.f90:117-151)
__device__ __forceinline__ lr nb_ratio(const FaceQ& f, lr ddx, lr ddy, lr ddu, lr ddv, lr zc) {
  const lr dn = ddx * f.xh + ddy * f.yh;
  const lr q = DIV(ddu * f.uh + ddv * f.vh, signF(maxF_nn(absF(dn), zc), dn));
#if BL_MIXED
  // FP32 saturates where FP64 would not: keep the ratio finite (the
  // limiter only distinguishes r below 0, in [0, 1] and above 1)
  return fmaxf(fminf(q * f.w1, 1e30f), -1e30f);
#else
  return q * f.w1;
#endif
}

// k_getdt of the fast build shares face work between neighbouring threads.
// A block of BS threads takes BS - 2 consecutive elements; thread t holds
// element blockIdx*(BS-2) + t - 1, so threads 0 and BS-1 hold the
// neighbours of the block's first and last elements (halos).  Every
// thread first publishes in shared memory the quantities of its face 0 and
// the differences of its faces 1 and 3; then each element takes
// - face 2 from the thread across it when that element is the adjacent one
//   and the face is its face 0 (the same edge run the other way: the
//   differences and unit vectors change sign, lengths and ratio do not);
// - the differences of a neighbour face of the limiter from the adjacent
//   thread when the neighbour is that element and the face is its face 1
//   or 3 (the same arithmetic on the same operands);
// and computes everything else itself, as the exact build does.  On the
// generated meshes elements are numbered along mesh lines, so the face
// across face 2 and the two limiter neighbours of side 0 are the adjacent
// elements and take the shared path.
// PART 0 is the whole kernel; with BL_GETDT_SPLIT the launch runs PART 1,
// the edge viscosity (elvisc and the corner forces), then PART 2, which
// reads elvisc back for the CFL and divergence candidates and the dt
// reduction (the same blocks over the same elements in both).
template <int BS, bool BATCH, int PART = 0>
__global__ void __launch_bounds__(BS, BL_GETDT_MINB) k_getdt(DevFields F, DevCfg C) {
  // the mesh of this block: the context's, or in a batch the block's own
  // (its blocks [blk0, blk0 + nblk), elements [el0, el1))
  DevStep* S = F.step;
  int blk0 = 0, nblk = (int)gridDim.x, el0 = 0, el1 = F.nel;
  const DevInst* I = nullptr;
  if (BATCH) {
    const int m = __ldg(F.blkinst + blockIdx.x);
    I = F.inst + m;
    S = F.steps + m;
    blk0 = I->blk_begin;
    nblk = I->blk_end - I->blk_begin;
    el0 = I->el_begin;
    el1 = I->el_end;
  }
  if (halted(S)) return;
  if (S->stop_next) {            // bl_run: the previous step reached time_end
    if ((int)blockIdx.x == blk0 && threadIdx.x == 0) S->halted = 1;
    return;
  }
  const int t = threadIdx.x;
  const int iel = el0 + ((int)blockIdx.x - blk0) * (BS - 2) + t - 1;
  const bool inmesh = iel >= el0 && iel < el1;
  const bool own = inmesh && t > 0 && t < BS - 1;
  double cflv = HUGE_VAL;        // sentinel above HUGE(1.0)
  int cfli = 0x7fffffff;
  double divv = DBL_MIN;         // TINY(1.0)
  int divi = -1;
  // face 0: du dv lu lx uh vh xh yh w1, then the edge coefficient's two
  // factors that do not depend on the side the face is seen from,
  // cvisc1*sqrt((cs2 + cs2')/2) + cvisc2*|du| and rho + rho' (the same sums
  // with the operands swapped, which IEEE addition does not change)
  __shared__ lr s_f0[11][BS];
  __shared__ lr s_fd[8][BS];  // faces 1, 3: dx dy du dv each
  const lr zl = lr_cut(C.zerocut);
  int n[4] = {0, 0, 0, 0};
  double x[4], y[4], u[4], v[4];
  if (inmesh) {
    const int4 nd = __ldg(F.ielnd + iel);
    n[0] = nd.x;
    n[1] = nd.y;
    n[2] = nd.z;
    n[3] = nd.w;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      x[j] = F.ndx[n[j]];
      y[j] = F.ndy[n[j]];
      u[j] = F.ndu[n[j]];
      v[j] = F.ndv[n[j]];
    }
  }
  if (PART != 2 && !C.ztq) {
    if (inmesh) {
      const FaceQ f0 = face_q(to_lr(u[1] - u[0]), to_lr(v[1] - v[0]), to_lr(x[1] - x[0]),
                              to_lr(y[1] - y[0]), zl);
      s_f0[0][t] = f0.du;
      s_f0[1][t] = f0.dv;
      s_f0[2][t] = f0.lu;
      s_f0[3][t] = f0.lx;
      s_f0[4][t] = f0.uh;
      s_f0[5][t] = f0.vh;
      s_f0[6][t] = f0.xh;
      s_f0[7][t] = f0.yh;
      s_f0[8][t] = f0.w1;
      const int nb0 = __ldg(F.ielel + iel).x;
      s_f0[9][t] = to_lr(C.cvisc1) * SQRT(to_lr(half(F.cs2[iel] + F.cs2[nb0]))) + to_lr(C.cvisc2) * f0.lu;
      s_f0[10][t] = to_lr(F.rho[iel] + F.rho[nb0]);
      s_fd[0][t] = to_lr(x[2] - x[1]);
      s_fd[1][t] = to_lr(y[2] - y[1]);
      s_fd[2][t] = to_lr(u[2] - u[1]);
      s_fd[3][t] = to_lr(v[2] - v[1]);
      s_fd[4][t] = to_lr(x[0] - x[3]);
      s_fd[5][t] = to_lr(y[0] - y[3]);
      s_fd[6][t] = to_lr(u[0] - u[3]);
      s_fd[7][t] = to_lr(v[0] - v[3]);
    }
    __syncthreads();
  }
  if (own) {
    const double rho0 = F.rho[iel];
    double visc = 0.0;
    if (PART != 2 && !C.ztq) {
      // hydro_kn_initeviscosity / limiteviscosity / geteviscosity
      // (hydro_kn_edgeviscosity.f90:30-282), face by face in the reference's
      // order 3, 1, 0, 2 (the faces of side s are (s+3)&3 and s+1)
      const int4 ee = __ldg(F.ielel + iel);
      const int nb[4] = {ee.x, ee.y, ee.z, ee.w};
      const int fcp = __ldg(F.ielfc + iel);
      const double cs2i = F.cs2[iel];
      // the vector from an edge's midpoint to the centroid is (a3,b3),
      // (-a1,-b1), (-a3,-b3), (a1,b1) for faces 0..3 (corners written as
      // s -+ a1 +- a2 -+ a3, exact in real arithmetic)
      const lr ga1 = to_lr(F.a1[iel]), ga3 = to_lr(F.a3[iel]), gb1 = to_lr(F.b1[iel]), gb3 = to_lr(F.b3[iel]);
      // |c|^2 of faces 1,3 and of faces 0,2 (only the cut test uses it)
      const lr c1sq = ga1 * ga1 + gb1 * gb1, c3sq = ga3 * ga3 + gb3 * gb3;
      // max over faces of edv * |du|; the reference's max of
      // edv * 2|du| / max(rho, zerocut) is that times 2 / max(rho, zerocut)
      lr vmax = (lr)0;
      lr edx[4], edy[4];
#pragma unroll
      for (int s = 0; s < 2; s++) {
        const int in1 = nb[s], in2 = nb[s + 2];
        const int f1 = fc_of(fcp, s), f2 = fc_of(fcp, s + 2);
        // boundary rule (hydro_kn_edgeviscosity.f90:154-183)
        lr val1 = (lr)0, val2 = (lr)0;
        if (in1 == iel)
          val1 = (__ldg(F.indtype + n[s]) < 0 && __ldg(F.indtype + n[(s + 1) & 3]) < 0 && in2 != iel)
                     ? (lr)1 : (lr)0;
        if (in2 == iel)
          val2 = (__ldg(F.indtype + n[s + 2]) < 0 && __ldg(F.indtype + n[(s + 3) & 3]) < 0 &&
                  in1 != iel) ? (lr)1 : (lr)0;
#pragma unroll
        for (int e2 = 0; e2 < 2; e2++) {
          const int is = e2 == 0 ? ((s + 3) & 3) : (s + 1);
          FaceQ f;
          int qf = -1;  // thread whose face-0 coefficient factors apply
          if (is == 0) {
            qf = t;
            f.du = s_f0[0][t];
            f.dv = s_f0[1][t];
            f.lu = s_f0[2][t];
            f.lx = s_f0[3][t];
            f.uh = s_f0[4][t];
            f.vh = s_f0[5][t];
            f.xh = s_f0[6][t];
            f.yh = s_f0[7][t];
            f.w1 = s_f0[8][t];
          } else if (is == 2) {
            const int o = nb[2] - iel;
            if ((o == 1 || o == -1) && fc_of(fcp, 2) == 0) {
              const int q = t + o;
              qf = q;
              f.du = negF(s_f0[0][q]);
              f.dv = negF(s_f0[1][q]);
              f.lu = s_f0[2][q];
              f.lx = s_f0[3][q];
              f.uh = negF(s_f0[4][q]);
              f.vh = negF(s_f0[5][q]);
              f.xh = negF(s_f0[6][q]);
              f.yh = negF(s_f0[7][q]);
              f.w1 = s_f0[8][q];
            } else {
              f = face_q(to_lr(u[3] - u[2]), to_lr(v[3] - v[2]), to_lr(x[3] - x[2]),
                         to_lr(y[3] - y[2]), zl);
            }
          } else {
            const int o = is == 1 ? 0 : 4;
            f = face_q(s_fd[o + 2][t], s_fd[o + 3][t], s_fd[o][t], s_fd[o + 1][t], zl);
          }
          // neighbour faces: edge 1 uses MOD(ielfc,4)+1 / MOD(ielfc+2,4)+1,
          // edge 2 the other pair (hydro_kn_edgeviscosity.f90:117-151)
          const int ins1 = e2 == 0 ? ((f1 + 1) & 3) : ((f1 + 3) & 3);
          const int ins2 = e2 == 0 ? ((f2 + 3) & 3) : ((f2 + 1) & 3);
          lr r1 = val1, r2 = val2;
#pragma unroll
          for (int k = 0; k < 2; k++) {
            const int inb = k == 0 ? in1 : in2;
            const int ins = k == 0 ? ins1 : ins2;
            if (inb == iel) continue;
            lr ddx, ddy, ddu, ddv;
            const int o = inb - iel;
            if ((o == 1 || o == -1) && (ins & 1)) {
              const int q = t + o, c = ins == 1 ? 0 : 4;
              ddx = s_fd[c][q];
              ddy = s_fd[c + 1][q];
              ddu = s_fd[c + 2][q];
              ddv = s_fd[c + 3][q];
            } else {
              const int4 m = __ldg(F.ielnd + inb);
              const int mm[4] = {m.x, m.y, m.z, m.w};
              const int a = mm[ins], b = mm[(ins + 1) & 3];
              ddx = to_lr(F.ndx[b] - F.ndx[a]);
              ddy = to_lr(F.ndy[b] - F.ndy[a]);
              ddu = to_lr(F.ndu[b] - F.ndu[a]);
              ddv = to_lr(F.ndv[b] - F.ndv[a]);
            }
            const lr r = nb_ratio(f, ddx, ddy, ddu, ddv, zl);
            if (k == 0) r1 = r;
            else r2 = r;
          }
          // limiter and edge coefficient (hydro_kn_edgeviscosity.f90:185-214)
          lr cq, rs;
          if (qf >= 0) {
            cq = s_f0[9][qf];
            rs = s_f0[10][qf];
          } else {
            const int ins = nb[is];
            cq = to_lr(C.cvisc1) * SQRT(to_lr(half(cs2i + F.cs2[ins]))) + to_lr(C.cvisc2) * f.lu;
            rs = to_lr(rho0 + F.rho[ins]);
          }
          lr w2 = minF(minF(minF(half(r1 + r2), twice(r1)), twice(r2)), (lr)1);
          w2 = maxF((lr)0, w2);
          const lr edv = half((lr)1 - w2) * rs * cq;
          vmax = maxF_nn(vmax, edv * f.lu);  // never negative
          // edge force (hydro_kn_edgeviscosity.f90:219-282): the reference
          // normalises the midpoint-to-centroid vector c, orients it by the
          // sign of its product with the face vector and scales it back by
          // |c|: (exh, eyh) = -+(cy, -cx), the sign bit of w33 = cy*xh -
          // cx*yh choosing; |c| only enters the cut test
          const lr cx = is == 0 ? ga3 : (is == 1 ? negF(ga1) : (is == 2 ? negF(ga3) : ga1));
          const lr cy = is == 0 ? gb3 : (is == 1 ? negF(gb1) : (is == 2 ? negF(gb3) : gb1));
          const lr w33 = cy * f.xh - cx * f.yh;
          const lr exh = negxorsign(cy, w33);
          const lr eyh = xorsign(cx, w33);
          const lr w7sq = (is & 1) ? c1sq : c3sq;
          const lr w6b = f.du * exh + f.dv * eyh;
          const lr d = edv * DIV(w6b, maxF_nn(f.lu, zl));
          edx[is] = f.du * d;
          edy[is] = f.dv * d;
          if (le_nn(f.lu, zl) || geF(zl, w6b) || le_nn(w7sq, zl * zl) || le_nn(f.lx, zl)) {
            edx[is] = (lr)0;
            edy[is] = (lr)0;
          }
        }
      }
      visc = from_lr(vmax * DIV((lr)2, maxF(to_lr(rho0), zl)));
      F.cnviscx[iel] = make_d4(from_lr(edx[0] - edx[3]), from_lr(edx[1] - edx[0]),
                               from_lr(edx[2] - edx[1]), from_lr(edx[3] - edx[2]));
      F.cnviscy[iel] = make_d4(from_lr(edy[0] - edy[3]), from_lr(edy[1] - edy[0]),
                               from_lr(edy[2] - edy[1]), from_lr(edy[3] - edy[2]));
      F.visc[iel] = visc;
    } else {
      visc = F.visc[iel];
    }
    if (PART != 1) getdt_tail(F, C, iel, x, y, u, v, visc, cflv, cfli, divv, divi);
  }
  if (PART != 1) getdt_finish<BS, BATCH>(F, C, S, cflv, cfli, divv, divi, blk0, nblk, el0, I);
}

template <int BS>
constexpr int getdt_elements_per_block() { return BS - 2; }
#else

template <int BS, bool BATCH, class L = DevLayout>
__global__ void __launch_bounds__(BS, BL_GETDT_MINB) k_getdt(DevFields F, DevCfg C) {
  // the mesh of this block: the context's, or in a batch the block's own
  // (its blocks [blk0, blk0 + nblk), elements [el0, el1))
  DevStep* S = F.step;
  int blk0 = 0, nblk = (int)gridDim.x, el0 = 0, el1 = F.nel;
  const DevInst* I = nullptr;
  if (BATCH) {
    const int m = __ldg(F.blkinst + blockIdx.x);
    I = F.inst + m;
    S = F.steps + m;
    blk0 = I->blk_begin;
    nblk = I->blk_end - I->blk_begin;
    el0 = I->el_begin;
    el1 = I->el_end;
  }
  if (halted(S)) return;
  if (S->stop_next) {            // bl_run: the previous step reached time_end
    if ((int)blockIdx.x == blk0 && threadIdx.x == 0) S->halted = 1;
    return;
  }
  const int iel = el0 + ((int)blockIdx.x - blk0) * BS + threadIdx.x;
  double cflv = HUGE_VAL;        // sentinel above HUGE(1.0)
  int cfli = 0x7fffffff;
  double divv = DBL_MIN;         // TINY(1.0)
  int divi = -1;
  if (iel < el1) {
    const int4 nd = L::nodes(F, iel);
    const int n[4] = {nd.x, nd.y, nd.z, nd.w};
    double x[4], y[4], u[4], v[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      x[j] = F.ndx[n[j]];
      y[j] = F.ndy[n[j]];
      u[j] = F.ndu[n[j]];
      v[j] = F.ndv[n[j]];
    }
    const double zc = C.zerocut;
    const double rho0 = F.rho[iel];
    double visc = 0.0;
    double qx[4] = {0.0, 0.0, 0.0, 0.0}, qy[4] = {0.0, 0.0, 0.0, 0.0};
    if (!C.ztq) {
      // hydro_kn_initeviscosity / limiteviscosity / geteviscosity
      // (hydro_kn_edgeviscosity.f90:30-282), evaluated face by face: every
      // quantity of a face -- its differences (face j runs corner j ->
      // j+1), lengths, normalised vectors, limiter ratios, edge coefficient
      // and edge force -- is formed and consumed before the next face, which
      // keeps the live state to the element's corners and the four edge
      // forces.  The faces of side s (neighbours across faces s and s+2)
      // are (s+3)&3 and s+1, in the reference's order 3, 1, 0, 2.
      const int4 ee = L::nbrs(F, iel);
      const int nb[4] = {ee.x, ee.y, ee.z, ee.w};
      const int fcp = L::faces(F, iel);
      const double cs2i = F.cs2[iel];
      const double xc = quarter(x[0] + x[1] + x[2] + x[3]);
      const double yc = quarter(y[0] + y[1] + y[2] + y[3]);
      double edx[4], edy[4];
#pragma unroll
      for (int s = 0; s < 2; s++) {
        const int in1 = nb[s], in2 = nb[s + 2];
        const int f1 = fc_of(fcp, s), f2 = fc_of(fcp, s + 2);
        // boundary rule (hydro_kn_edgeviscosity.f90:154-183): a ratio across
        // a boundary face is 1 between two boundary nodes facing an
        // interior neighbour, 0 otherwise
        double val1 = 0.0, val2 = 0.0;
        if (in1 == iel)
          val1 = (__ldg(F.indtype + n[s]) < 0 && __ldg(F.indtype + n[(s + 1) & 3]) < 0 && in2 != iel)
                     ? 1.0 : 0.0;
        if (in2 == iel)
          val2 = (__ldg(F.indtype + n[s + 2]) < 0 && __ldg(F.indtype + n[(s + 3) & 3]) < 0 &&
                  in1 != iel) ? 1.0 : 0.0;
#pragma unroll
        for (int e2 = 0; e2 < 2; e2++) {
          const int is = e2 == 0 ? ((s + 3) & 3) : (s + 1);
          const int jn = (is + 1) & 3;
          double w1 = u[jn] - u[is], w2 = v[jn] - v[is];
          double w3 = x[jn] - x[is], w4 = y[jn] - y[is];
          const double du = w1, dv = w2;
          double den = SQRT(w1 * w1 + w2 * w2);
          const double lu = den;
          den = DIV(1.0, maxF_nn(den, zc));
          const double uhat = w1 * den, vhat = w2 * den;
          den = SQRT(w3 * w3 + w4 * w4);
          const double lx = den;
          den = DIV(1.0, maxF_nn(den, zc));
          const double xh = w3 * den, yh = w4 * den;
          den = w3 * xh + w4 * yh;
          w1 = DIV(w1 * uhat + w2 * vhat, signF(maxF_nn(absF(den), zc), den));
          w1 = DIV(1.0, signF(maxF_nn(absF(w1), zc), w1));
          // neighbour faces: edge 1 uses MOD(ielfc,4)+1 / MOD(ielfc+2,4)+1,
          // edge 2 the other pair (hydro_kn_edgeviscosity.f90:117-151)
          const int ins1 = e2 == 0 ? ((f1 + 1) & 3) : ((f1 + 3) & 3);
          const int ins2 = e2 == 0 ? ((f2 + 3) & 3) : ((f2 + 1) & 3);
          double r1 = val1, r2 = val2;
          if (in1 != iel) {
            const int4 m = L::nodes(F, in1);
            const int mm[4] = {m.x, m.y, m.z, m.w};
            const int a = mm[ins1], b = mm[(ins1 + 1) & 3];
            double ddx = F.ndx[b] - F.ndx[a], ddy = F.ndy[b] - F.ndy[a];
            double ddu = F.ndu[b] - F.ndu[a], ddv = F.ndv[b] - F.ndv[a];
            double dn = ddx * xh + ddy * yh;
            double q = DIV(ddu * uhat + ddv * vhat, signF(maxF_nn(absF(dn), zc), dn));
            r1 = q * w1;
          }
          if (in2 != iel) {
            const int4 m = L::nodes(F, in2);
            const int mm[4] = {m.x, m.y, m.z, m.w};
            const int a = mm[ins2], b = mm[(ins2 + 1) & 3];
            double ddx = F.ndx[b] - F.ndx[a], ddy = F.ndy[b] - F.ndy[a];
            double ddu = F.ndu[b] - F.ndu[a], ddv = F.ndv[b] - F.ndv[a];
            double dn = ddx * xh + ddy * yh;
            double q = DIV(ddu * uhat + ddv * vhat, signF(maxF_nn(absF(dn), zc), dn));
            r2 = q * w1;
          }
          // limiter and edge coefficient (hydro_kn_edgeviscosity.f90:185-214)
          const int ins = nb[is];
          w1 = C.cvisc1 * SQRT(half(cs2i + F.cs2[ins]));
          w2 = r1;
          w3 = r2;
          w2 = minF(minF(minF(half(w2 + w3), twice(w2)), twice(w3)), 1.0);
          w2 = maxF(0.0, w2);
          w4 = lu;
          w3 = half(1.0 - w2) * (rho0 + F.rho[ins]) * (w1 + C.cvisc2 * w4);
          const double edv = w3;
          w4 = DIV(twice(w4), maxF(rho0, zc));
          visc = maxF_nn(visc, w3 * w4);  // visc stays +0 or positive
          // edge force (hydro_kn_edgeviscosity.f90:219-282)
          {
            const double m3 = half(x[is] + x[jn]);
            const double m6 = half(y[is] + y[jn]);
            const double w7 = SQRT((xc - m3) * (xc - m3) + (yc - m6) * (yc - m6));
            const double w8 = lx;  // SQRT(w1*w1+w4*w4) of the same face difference
            double d = DIV(1.0, w7);
            double exh = (yc - m6) * d, eyh = (m3 - xc) * d;
            // w1*(1/w8), w4*(1/w8): the limiter's normalised face vector
            // whenever w8 > zerocut; otherwise the edge is cut below
            const double w33 = exh * xh + eyh * yh;
            d = -(signF(1.0, w33) * w7);
            exh = exh * d;
            eyh = eyh * d;
            const double w5 = lu;
            const double w6b = du * exh + dv * eyh;
            d = DIV(w6b, maxF_nn(w5, zc));
            edx[is] = edv * du * d;
            edy[is] = edv * dv * d;
            if (le_nn(w5, zc) || geF(zc, w6b) || le_nn(w7, zc) || le_nn(w8, zc)) {
              edx[is] = 0.0;
              edy[is] = 0.0;
            }
          }
        }
      }
      qx[0] = edx[0] - edx[3];
      qx[1] = edx[1] - edx[0];
      qx[2] = edx[2] - edx[1];
      qx[3] = edx[3] - edx[2];
      qy[0] = edy[0] - edy[3];
      qy[1] = edy[1] - edy[0];
      qy[2] = edy[2] - edy[1];
      qy[3] = edy[3] - edy[2];
      L::corners(F.cnviscx, iel, qx);
      L::corners(F.cnviscy, iel, qy);
      F.visc[iel] = visc;
    } else {
      visc = F.visc[iel];
    }
    getdt_tail<L>(F, C, iel, x, y, u, v, visc, cflv, cfli, divv, divi);
  }
  getdt_finish<BS, BATCH>(F, C, S, cflv, cfli, divv, divi, blk0, nblk, el0, I);
}

template <int BS>
constexpr int getdt_elements_per_block() { return BS; }
#endif

// ================================================================ k_lag_force

template <int BS, bool BATCH>
__global__ void __launch_bounds__(BS, BL_FORCE_MINB) k_lag_force(DevFields F, DevCfg C) {
  const int iel = blockIdx.x * BS + threadIdx.x;
  if (iel >= F.nel) return;
  DevStep* S = el_step<BATCH>(F, iel);
  if (halted(S)) return;
  const double dt = S->dt;
  const double hdt = 0.5 * dt;   // time_dr_setpredictor dts / getvertex step
  const double zc = C.zerocut;
  const int4 nd = __ldg(F.ielnd + iel);
  const int n[4] = {nd.x, nd.y, nd.z, nd.w};
  double x[4], y[4], u[4], v[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    x[j] = F.ndx[n[j]];
    y[j] = F.ndy[n[j]];
    u[j] = F.ndu[n[j]];
    v[j] = F.ndv[n[j]];
  }
  const d4 qx = F.cnviscx[iel], qy = F.cnviscy[iel];
  const int ireg = __ldg(F.ielreg + iel);
  const int mat = __ldg(F.ielmat + iel);
  const double m = F.mass[iel];
  const double e0 = F.e[iel];
  const int imx = F.elmx ? F.elmx[iel] : -1;
  double fx[4], fy[4];
  // ---- predictor force at t^n (hydro_dr_getforce, zcorrector false)
  const double a1 = F.a1[iel], a3 = F.a3[iel], b1 = F.b1[iel], b3 = F.b3[iel];
  force_pq(F.p[iel], a1, a3, b1, b3, qx, qy, fx, fy);
  if (C.zsp) {
#if BL_FAST_ALGEBRA
    const double a2 = F.a2[iel], b2 = F.b2[iel];
    const double cross = a1 * b3 - a3 * b1;
    const double t1 = a1 * b2 - a2 * b1, t3 = a3 * b2 - a2 * b3;
    force_sp_iso(__ldg(C.pmeritreg + ireg), F.rho[iel], F.cs2v[iel], cross, t1 + t3, t3 - t1, a1,
                 a2, a3, b1, b2, b3, F.spmass[iel], fx, fy);
#else
    force_sp(__ldg(C.pmeritreg + ireg), F.rho[iel], F.cs2v[iel], x, y, F.spmass[iel], fx, fy);
#endif
  }
  // ---- half-step vertices (geometry_kn_getvertex with 0.5*dt)
  double xh[4], yh[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    xh[j] = x[j] + hdt * u[j];
    yh[j] = y[j] + hdt * v[j];
  }
  // ---- geometry, density (geometry_dr_getgeometry, density_dr_getdensity)
  Iso g = getiso(xh, yh);
  if (gtF(0.0, g.vol)) atomicMax(&S->negvol_pred, iel + 1 - el_base<BATCH>(F, iel));
  const double rho = DIV(m, g.vol);
  // ---- energy (hydro_kn_getenergy with dts = dt/2) and EoS
  const double eh = energy_update(e0, m, zc, hdt, fx, fy, u, v);
  double ph, cs2h;
  eos_pc(C, mat, rho, eh, ph, cs2h);
  // ---- mixed cells: component state at the half step
  if (imx >= 0) {
    const int c0 = F.imxfcp[imx], nc = F.imxncp[imx];
    double ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0};
    for (int k = 0; k < nc; k++) {
      const int icp = c0 + k;
      const double fr = F.frvol[icp];
      // predictor component force with the t^n component state
      double cfx[4], cfy[4];
      force_pq(F.cpp[icp], a1, a3, b1, b3, F.cpviscx[icp],
               F.cpviscy[icp], cfx, cfy);
      // component energy with cpu = frvolume*cnu (utils_kn_mxgathercnav)
      double cu[4], cv[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        cu[j] = fr * u[j];
        cv[j] = fr * v[j];
      }
      const double cpm = F.cpm[icp];
      const double cpe = energy_update(F.cpe[icp], cpm, zc, hdt, cfx, cfy, cu, cv);
      F.cpe[icp] = cpe;  // the reference does not restore component energy
      const double cpv = times4(g.a1 * g.b3 - g.a3 * g.b1) * fr;
      const double cpr = DIV(cpm, cpv);
      double cpp, cpc;
      eos_pc(C, __ldg(F.icpmat + icp), cpr, cpe, cpp, cpc);
      // corrector component force at the half-step state
      force_pq(cpp, g.a1, g.a3, g.b1, g.b3, F.cpviscx[icp], F.cpviscy[icp], cfx, cfy);
      F.cpfx[icp] = make_d4(cfx[0], cfx[1], cfx[2], cfx[3]);
      F.cpfy[icp] = make_d4(cfy[0], cfy[1], cfy[2], cfy[3]);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        ax[j] = ax[j] + fr * cfx[j];
        ay[j] = ay[j] + fr * cfy[j];
      }
    }
    // corrector element force: P+Q+SP+HG are overwritten by the average
#pragma unroll
    for (int j = 0; j < 4; j++) {
      fx[j] = ax[j];
      fy[j] = ay[j];
    }
  } else {
    // ---- corrector force at the half step (zcorrector true)
    force_pq(ph, g.a1, g.a3, g.b1, g.b3, qx, qy, fx, fy);
    if (C.zsp) {
#if BL_FAST_ALGEBRA
      force_sp_iso(__ldg(C.pmeritreg + ireg), rho, cs2h, g.cross, g.ts, g.td, g.a1, g.a2, g.a3,
                   g.b1, g.b2, g.b3, F.spmass[iel], fx, fy);
#else
      force_sp(__ldg(C.pmeritreg + ireg), rho, cs2h, xh, yh, F.spmass[iel], fx, fy);
#endif
    }
    if (C.zhg) force_hg(__ldg(C.kappareg + ireg), rho, g.vol, S->rdt, u, v, fx, fy);
  }
  F.cnfx[iel] = make_d4(fx[0], fx[1], fx[2], fx[3]);
  F.cnfy[iel] = make_d4(fy[0], fy[1], fy[2], fy[3]);
  F.rho_h[iel] = rho;
  F.cnwt_h[iel] = make_d4(g.w0, g.w1, g.w2, g.w3);
}

// ================================================================ k_lag_accel

template <int BS, bool BATCH>
__global__ void BL_ACCEL_BOUNDS(BS) k_lag_accel(DevFields F, DevCfg C) {
  const int ind = blockIdx.x * BS + threadIdx.x;
  if (ind >= F.nnd) return;
  const DevStep* S = nd_step<BATCH>(F, ind);
  if (halted(S)) return;
  const double dt = S->dt;
  const double zc = C.zerocut;
  // hydro_kn_scatteracceleration: corner-major order over ielsort
  double ndm = 0.0, nda = 0.0, fx = 0.0, fy = 0.0;
  const int b = __ldg(F.nc_off + ind), e = __ldg(F.nc_off + ind + 1);
  for (int k = b; k < e; k++) {
    const int c = __ldg(F.nc_ent + k);
    const int iel = c >> 2, jj = c & 3;
    const double* cm = reinterpret_cast<const double*>(F.cnmass + iel);
    const double cmj = cm[jj];
    const double cw = reinterpret_cast<const double*>(F.cnwt_h + iel)[jj];
    if (gtF(cmj, zc)) {
      ndm = ndm + cmj;
    } else {
      const double cmi = cm[(jj + 3) & 3];
      if (gtF(cmi, zc)) ndm = ndm + cmi;
      else ndm = ndm + F.rho_h[iel] * cw;
    }
    nda = nda + cw;
    fx = fx + reinterpret_cast<const double*>(F.cnfx + iel)[jj];
    fy = fy + reinterpret_cast<const double*>(F.cnfy + iel)[jj];
  }
  // hydro_kn_getacceleration
  const double w1 = C.dencut * nda;
  double ax, ay;
  if (gtF(ndm, w1)) {
    ax = DIV(fx, ndm);
    ay = DIV(fy, ndm);
  } else {
    ax = 0.0;
    ay = 0.0;
  }
  // utils_kn_bc on the accelerations
  const int t = __ldg(F.indtype + ind);
  if (t == -1) ax = 0.0;
  else if (t == -2) ay = 0.0;
  else if (t == -3) { ax = 0.0; ay = 0.0; }
  const double w2 = ax * ax + ay * ay;
  if (gt_nn(C.accut * C.accut, w2)) {  // w2 is a sum of squares
    ax = 0.0;
    ay = 0.0;
  }
  // hydro_kn_applyacceleration, then both half vertex moves
  const double hdt = 0.5 * dt;
  const double u0 = F.ndu[ind], v0 = F.ndv[ind];
  const double u1 = u0 + dt * ax, v1 = v0 + dt * ay;
  const double ub = u0 + hdt * ax, vb = v0 + hdt * ay;
  double x = F.ndx[ind], y = F.ndy[ind];
  x = x + hdt * u0;
  y = y + hdt * v0;
  x = x + hdt * u1;
  y = y + hdt * v1;
  F.ndu[ind] = u1;
  F.ndv[ind] = v1;
  F.ndubar[ind] = ub;
  F.ndvbar[ind] = vb;
  F.ndx[ind] = x;
  F.ndy[ind] = y;
}

// ================================================================ k_lag_state

template <int BS, bool BATCH>
__global__ void BL_STATE_BOUNDS(BS) k_lag_state(DevFields F, DevCfg C) {
  const int iel = blockIdx.x * BS + threadIdx.x;
  if (iel >= F.nel) return;
  DevStep* S = el_step<BATCH>(F, iel);
  if (halted(S)) return;
  const double dt = S->dt;
  const double zc = C.zerocut;
  const int4 nd = __ldg(F.ielnd + iel);
  const int n[4] = {nd.x, nd.y, nd.z, nd.w};
  double x[4], y[4], ub[4], vb[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    x[j] = F.ndx[n[j]];
    y[j] = F.ndy[n[j]];
    ub[j] = F.ndubar[n[j]];
    vb[j] = F.ndvbar[n[j]];
  }
  Iso g = getiso(x, y);
  if (gtF(0.0, g.vol)) atomicMax(&S->negvol_corr, iel + 1 - el_base<BATCH>(F, iel));
  const double m = F.mass[iel];
  const double rho = DIV(m, g.vol);
  const d4 f4x = F.cnfx[iel], f4y = F.cnfy[iel];
  const double fx[4] = {f4x.x, f4x.y, f4x.z, f4x.w};
  const double fy[4] = {f4y.x, f4y.y, f4y.z, f4y.w};
  const double e = energy_update(F.e[iel], m, zc, dt, fx, fy, ub, vb);
  double p, cs2;
  eos_pc(C, __ldg(F.ielmat + iel), rho, e, p, cs2);
  F.a1[iel] = g.a1;
  F.a2[iel] = g.a2;
  F.a3[iel] = g.a3;
  F.b1[iel] = g.b1;
  F.b2[iel] = g.b2;
  F.b3[iel] = g.b3;
  F.cnwt[iel] = make_d4(g.w0, g.w1, g.w2, g.w3);
  const int imx = F.elmx ? F.elmx[iel] : -1;
  // the learned closure (k_mix_closure, launched next) splits a two-material
  // cell's volume change between its materials and updates them: it needs
  // the cell volume at the start of the step
  const bool learned = imx >= 0 && F.closure && F.imxncp[imx] == 2;
  if (learned) F.mxv0[imx] = F.vol[iel];
  F.vol[iel] = g.vol;
  F.rho[iel] = rho;
  F.e[iel] = e;
  F.p[iel] = p;
  F.cs2[iel] = cs2;
  if (imx >= 0 && !learned) {
    const int c0 = F.imxfcp[imx], nc = F.imxncp[imx];
    for (int k = 0; k < nc; k++) {
      const int icp = c0 + k;
      const double fr = F.frvol[icp];
      const d4 a = F.cpfx[icp], b = F.cpfy[icp];
      const double cfx[4] = {a.x, a.y, a.z, a.w}, cfy[4] = {b.x, b.y, b.z, b.w};
      double cu[4], cv[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        cu[j] = fr * ub[j];
        cv[j] = fr * vb[j];
      }
      const double cpm = F.cpm[icp];
      const double cpe = energy_update(F.cpe[icp], cpm, zc, dt, cfx, cfy, cu, cv);
      const double cpv = times4(g.a1 * g.b3 - g.a3 * g.b1) * fr;
      const double cpr = DIV(cpm, cpv);
      double cpp, cpc;
      eos_pc(C, __ldg(F.icpmat + icp), cpr, cpe, cpp, cpc);
      F.cpe[icp] = cpe;
      F.cpvol[icp] = cpv;
      F.cprho[icp] = cpr;
      F.cpp[icp] = cpp;
      F.cpcs2[icp] = cpc;
    }
  }
}

// ================================================================ k_mix_closure

// The learned mixed-cell closure, after k_lag_state.  For each two-material
// cell the network (tensor cores, 16 cells per warp) predicts the volume
// each material gains over the step beyond the plain closure's share (its
// volume fraction of the cell's change), as a fraction of the cell's volume
// at the start: x_m = norm[20] * y_m.  Its inputs, standardised as
// (f - norm[k]) * norm[10 + k], are the state at the start of the step:
//   0 material 1's volume fraction, 1-2 the densities, 3-4 the pressures,
//   5-6 the sound speeds squared, 7 dV / V^n, 8 dt sqrt(max cs2 / V^n) (a
//   Courant number of the cell), 9 (p1 - p2) / (|p1| + |p2|).
// The exchange used is x = (x_1 - x_2) / 2 into material 1 (x_1 + x_2 = 0
// conserves the cell's volume), limited to the admissible range between 0
// and x_eq, the exchange that equalises the two materials' pressures after
// the plain closure's step (linearised with the bulk moduli rho c^2): the
// closure may relax the materials towards pressure equilibrium, not past it.
// The plain closure is kept in a cell whose outputs are not finite, miss
// conservation (|y_1 + y_2| > norm[21]), lie out of range (farther than
// |x_eq| outside [0, x_eq]) or leave a material a non-positive volume;
// F.mlp_count[1] counts those cells.  Each material's energy takes the plain
// closure's work; with F.closure == 1 the exchanged volume also trades
// energy at the mixture pressure fr_1 p_1 + fr_2 p_2 (the work one material
// does on the other, summing to zero over the cell), with F.closure == 2
// the materials keep their specific energies, so that for ideal gases the
// cell's mixture pressure sum (gamma_m - 1) E_m / V, and with it every later
// element and node field, stays the plain closure's.  Either way the cell's
// volume and total energy, and every element and node field of the step,
// are the plain closure's, and a rejected cell ends exactly as under it.
// In a batch each cell reads the step header of its own mesh.
constexpr int kClosureWarps = 4;
template <bool BATCH>
__global__ void __launch_bounds__(32 * kClosureWarps) k_mix_closure(DevFields F, DevCfg C) {
  if (!BATCH && halted(F.step)) return;
  extern __shared__ unsigned char smem[];
  mlp::SmemW& w = *reinterpret_cast<mlp::SmemW*>(smem);
  mlp::SmemS* Ss = reinterpret_cast<mlp::SmemS*>(smem + sizeof(mlp::SmemW));
  mlp::copy_weights<32 * kClosureWarps>(w, F.mlp_img);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  mlp::SmemS& s = Ss[warp];
  const int imx = blockIdx.x * (16 * kClosureWarps) + warp * 16 + (lane & 15);
  // lanes l and l + 16 share cell l: the features and the network take one
  // row per cell (lanes 0-15), the FP64 update one material per lane
  const int k = lane >> 4;
  const bool two = imx < F.nmx && F.imxncp[imx] == 2;
  const int iel = two ? F.imxel[imx] : 0;
  const DevStep* S = el_step<BATCH>(F, iel);
  const bool cell = two && !halted(S);
  const double dt = cell ? S->dt : 0.0;
  double V0 = 0.0, V1 = 0.0;
  int c0 = 0;
  if (cell) {
    c0 = F.imxfcp[imx];
    V0 = F.mxv0[imx];
    V1 = F.vol[iel];
  }
  if (lane < 16) {
    float f[mlp::NI];
    if (cell) {
      const double p1 = F.cpp[c0], p2 = F.cpp[c0 + 1];
      const double q1 = F.cpcs2[c0], q2 = F.cpcs2[c0 + 1];
      const double raw[mlp::NI] = {F.frvol[c0], F.cprho[c0], F.cprho[c0 + 1], p1, p2, q1, q2,
                                   (V1 - V0) / V0, dt * sqrt(maxF(q1, q2) / V0),
                                   (p1 - p2) / (absF(p1) + absF(p2) + 1e-300)};
#pragma unroll
      for (int j = 0; j < mlp::NI; j++)
        f[j] = ((float)raw[j] - __ldg(F.mlp_norm + j)) * __ldg(F.mlp_norm + mlp::NI + j);
    }
#pragma unroll
    for (int j = 0; j < 16; j++) s.x[lane][j] = (cell && j < mlp::NI) ? f[j] : 0.0f;
  }
  __syncwarp();
  mlp::forward_warp(w, s);
  // this lane's material: the plain closure's step (k_lag_state's component
  // update), the fallback and the state the admissible range is measured from
  const double zc = C.zerocut;
  const int icp = c0 + k;
  double fr[2] = {0.0, 0.0}, pbar = 0.0;
  double pe = 0.0, pv = 0.0, pr = 0.0, pp = 0.0, pc = 0.0;
  if (cell) {
    fr[0] = F.frvol[c0];
    fr[1] = F.frvol[c0 + 1];
    pbar = fr[0] * F.cpp[c0] + fr[1] * F.cpp[c0 + 1];
    const double frk = k ? fr[1] : fr[0];
    const int4 nd = __ldg(F.ielnd + iel);
    const int n[4] = {nd.x, nd.y, nd.z, nd.w};
    const d4 a = F.cpfx[icp], b = F.cpfy[icp];
    const double cfx[4] = {a.x, a.y, a.z, a.w}, cfy[4] = {b.x, b.y, b.z, b.w};
    double cu[4], cv[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      cu[j] = frk * F.ndubar[n[j]];
      cv[j] = frk * F.ndvbar[n[j]];
    }
    const double cpm = F.cpm[icp];
    pe = energy_update(F.cpe[icp], cpm, zc, dt, cfx, cfy, cu, cv);
    pv = V1 * frk;
    pr = DIV(cpm, pv);
    eos_pc(C, __ldg(F.icpmat + icp), pr, pe, pp, pc);
  }
  // the other material's, from the partner lane
  const double opp = __shfl_xor_sync(0xffffffffu, pp, 16);
  const double opr = __shfl_xor_sync(0xffffffffu, pr, 16);
  const double opc = __shfl_xor_sync(0xffffffffu, pc, 16);
  if (!cell) return;
  const double P0 = k ? opp : pp, P1 = k ? pp : opp;
  const double R0 = k ? opr : pr, R1 = k ? pr : opr;
  const double Q0 = k ? opc : pc, Q1 = k ? pc : opc;
  const double xeq = DIV((P0 - P1) * V1, V0 * (DIV(R0 * Q0, fr[0]) + DIV(R1 * Q1, fr[1])));
  const double lo = fmin(0.0, xeq), hi = fmax(0.0, xeq), m = absF(xeq);
  const float o1 = s.y[lane & 15][0], o2 = s.y[lane & 15][1];
  const double xp = 0.5 * __ldg(F.mlp_norm + 2 * mlp::NI) * ((double)o1 - (double)o2);
  const double xm = fmin(fmax(xp, lo), hi);
  const double xk = k ? -xm : xm;  // this lane's material's share of the exchange
  const bool ok = isfinite(o1) && isfinite(o2) && isfinite(xeq) &&
                  fabsf(o1 + o2) <= __ldg(F.mlp_norm + 2 * mlp::NI + 1) && xp >= lo - m &&
                  xp <= hi + m && V1 * fr[0] + xm * V0 > 0.0 && V1 * fr[1] + (-xm) * V0 > 0.0;
  if (k == 0) {
    atomicAdd(F.mlp_count, 1ull);
    if (!ok) atomicAdd(F.mlp_count + 1, 1ull);
  }
  double cpv = pv, cpe = pe, cpr = pr, cpp = pp, cpc = pc;
  if (ok) {
    const double cpm = F.cpm[icp];
    cpv = pv + xk * V0;
    if (F.closure == 1) cpe = pe - DIV(pbar * (xk * V0), maxF(cpm, zc));
    cpr = DIV(cpm, cpv);
    eos_pc(C, __ldg(F.icpmat + icp), cpr, cpe, cpp, cpc);
    F.frvol[icp] = DIV(cpv, V1);
  }
  F.cpe[icp] = cpe;
  F.cpvol[icp] = cpv;
  F.cprho[icp] = cpr;
  F.cpp[icp] = cpp;
  F.cpcs2[icp] = cpc;
}

// ================================================================ launchers

static constexpr int BS_DT = 128;
static constexpr int BS_EL = 128;
static constexpr int BS_ND = 256;

// one block per getdt_elements_per_block elements
int getdt_blocks(int nel) {
  constexpr int E = getdt_elements_per_block<BS_DT>();
  return (nel + E - 1) / E;
}

// a single mesh's grid and number of partials: the same blocks (an equal
// share per block over whole resident waves was measured slower: the SMs'
// spread of finishing times is a spread of their speeds, not of their work)
int getdt_grid(int nel) { return getdt_blocks(nel); }

int getdt_launches(const DevCfg& C) {
#if BL_FAST_ALGEBRA && BL_GETDT_SPLIT
  return C.ztq ? 1 : 2;
#else
  (void)C;
  return 1;
#endif
}
void launch_getdt(const DevFields& F, const DevCfg& C, cudaStream_t s) {
#if BL_FAST_ALGEBRA && BL_GETDT_SPLIT
  if (!C.ztq) k_getdt<BS_DT, false, 1><<<getdt_grid(F.nel), BS_DT, 0, s>>>(F, C);
  k_getdt<BS_DT, false, 2><<<getdt_grid(F.nel), BS_DT, 0, s>>>(F, C);
#else
  k_getdt<BS_DT, false><<<getdt_grid(F.nel), BS_DT, 0, s>>>(F, C);
#endif
}
void launch_lag_force(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  k_lag_force<BS_EL, false><<<(F.nel + BS_EL - 1) / BS_EL, BS_EL, 0, s>>>(F, C);
}
void launch_lag_accel(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  k_lag_accel<BS_ND, false><<<(F.nnd + BS_ND - 1) / BS_ND, BS_ND, 0, s>>>(F, C);
}
void launch_lag_state(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  k_lag_state<BS_EL, false><<<(F.nel + BS_EL - 1) / BS_EL, BS_EL, 0, s>>>(F, C);
}
constexpr size_t kClosureSmem = sizeof(mlp::SmemW) + kClosureWarps * sizeof(mlp::SmemS);
int prepare_mix_closure() {
  return cudaFuncSetAttribute(k_mix_closure<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kClosureSmem) == cudaSuccess &&
                 cudaFuncSetAttribute(k_mix_closure<true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kClosureSmem) == cudaSuccess
             ? 0 : -1;
}
void launch_mix_closure(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  if (!F.closure || F.nmx < 1) return;
  const int per = 16 * kClosureWarps;
  k_mix_closure<false><<<(F.nmx + per - 1) / per, 32 * kClosureWarps, kClosureSmem, s>>>(F, C);
}
void launch_mix_closure_batch(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  if (!F.closure || F.nmx < 1) return;
  const int per = 16 * kClosureWarps;
  k_mix_closure<true><<<(F.nmx + per - 1) / per, 32 * kClosureWarps, kClosureSmem, s>>>(F, C);
}
// a batch of meshes: k_getdt over each mesh's own blocks, the rest over all
// elements or nodes, each reading the step header of its mesh
void launch_getdt_batch(const DevFields& F, const DevCfg& C, cudaStream_t s) {
#if BL_FAST_ALGEBRA && BL_GETDT_SPLIT
  if (!C.ztq) k_getdt<BS_DT, true, 1><<<F.nblk_batch, BS_DT, 0, s>>>(F, C);
  k_getdt<BS_DT, true, 2><<<F.nblk_batch, BS_DT, 0, s>>>(F, C);
#else
  k_getdt<BS_DT, true><<<F.nblk_batch, BS_DT, 0, s>>>(F, C);
#endif
}
void launch_lag_force_batch(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  k_lag_force<BS_EL, true><<<(F.nel + BS_EL - 1) / BS_EL, BS_EL, 0, s>>>(F, C);
}
void launch_lag_accel_batch(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  // block size chosen by the batch's autotuner (128, 256 or 512)
  if (F.nd_block == 128) k_lag_accel<128, true><<<(F.nnd + 127) / 128, 128, 0, s>>>(F, C);
  else if (F.nd_block == 512) k_lag_accel<512, true><<<(F.nnd + 511) / 512, 512, 0, s>>>(F, C);
  else k_lag_accel<256, true><<<(F.nnd + 255) / 256, 256, 0, s>>>(F, C);
}
void launch_lag_state_batch(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  k_lag_state<BS_EL, true><<<(F.nel + BS_EL - 1) / BS_EL, BS_EL, 0, s>>>(F, C);
}

}  // namespace BL_NS
}  // namespace bl
