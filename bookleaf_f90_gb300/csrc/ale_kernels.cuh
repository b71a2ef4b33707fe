// ale_kernels.cu -- the Eulerian remap (adv_type 1, isotropic) on sm_103a.
//
// Four kernels per ALE step replace the reference's loops of
// inf_solver_alestep (inf_solver_alestep.f90:39-74):
//   k_ale_flux    ale_kn_getmeshvelocity + geometry_kn_getvertex +
//                 geometry_kn_getfluxvolume (flux volume of every face; the
//                 neighbour's value for a shared face is minus the own one
//                 before the cut, so the volume sum needs no second pass),
//                 ale_kn_sumflux(fcdv) and the mass flux ale_kn_fluxelvl.
//   k_ale_el      ale_kn_sumflux(fcdm), ale_kn_updatebasisel, the energy flux
//                 ale_kn_fluxelvl, ale_kn_fluxbasisnd (corner mass fluxes)
//                 and both momentum passes of ale_kn_fluxndvl.
//   k_ale_nd      per node: ale_kn_calcbasisnd, massbasisnd, cutbasisnd,
//                 activend and both ale_kn_updatend passes, as CSR gathers in
//                 the reference's element-major order; writes the remapped
//                 vertices (the Eulerian mesh).
//   k_ale_update  ale_kn_updateel (energy), then ale_dr_hydroupdate
//                 (geometry, density, EoS) and the new corner masses.
#pragma once
#include <cfloat>
#include <cmath>

#include "bl_device.cuh"
#include "bl_kernels.h"

namespace bl {
namespace BL_NS {

__device__ __forceinline__ bool halted_a(const DevStep* S) {
  return *((volatile const int*)&S->halted) != 0;
}

// ale_active (ale_dr_utils.f90:35-51)
__device__ __forceinline__ bool ale_on(const DevCfg& C, const DevStep* S) {
  if (!C.ale_zexist) return false;
  const double t = S->time;
  return geF(t, C.ale_mintime) && geF(C.ale_maxtime, t);  // the IEEE >= on the integer pipe
}

__device__ __forceinline__ double cget(const d4* a, int iel, int j) {
  return reinterpret_cast<const double*>(a + iel)[j];
}

// geometry_kn_getfluxvolume for one face (before the cut)
__device__ __forceinline__ double face_dv(double x1, double x2, double y1, double y2, double x3,
                                          double x4, double y3, double y4) {
  double a1 = (-x1 - x4) + (x3 + x2);
  double a3 = (-x1 + x4) + (x3 - x2);
  double b1 = (-y1 - y4) + (y3 + y2);
  double b3 = (-y1 + y4) + (y3 - y2);
  return quarter(a1 * b3 - a3 * b1);
}

// w7 * m with w7 = SIGN(1, w) and m >= 0, and the test w1 * w2 <= 0 of the
// limiters.  The fast build takes the sign bit instead of the product (the
// same in real arithmetic: opposite signs or a zero), the exact build
// evaluates them as written.
__device__ __forceinline__ double sign_of(double m, double w) {
#if BL_FAST_ALGEBRA
  return signF(m, w);
#else
  return signF(1.0, w) * m;
#endif
}
__device__ __forceinline__ bool prod_le0(double w1, double w2) {
#if BL_FAST_ALGEBRA
  const long long b1 = bits64(w1), b2 = bits64(w2);
  return (b1 ^ b2) < 0 || (b1 << 1) == 0 || (b2 << 1) == 0;
#else
  return geF(0.0, w1 * w2);
#endif
}

#if BL_MIXED
// Mixed build: the remap limiters' gradient in FP32.  For the differences
// A, B of the advected variable towards the two neighbours and the masses
// (or volumes) mA, mB of the two sides, w8 = (A mB^2 + B mA^2) /
// (mA mB (mA + mB)) and |grad| = min(|w8|, |A|/mA, |B|/mB), zero unless A
// and B have the same sign, with the sign of S.  The operands are brought
// into FP32's range by powers of two taken from their exponents (exact),
// and the result scaled back, all on the integer pipe (f32_of, f64_of).
__device__ __forceinline__ int exp_of(double x) {
  return (int)((bits64(x) >> 52) & 0x7ff) - 1023;
}
__device__ __forceinline__ double grad_f32(double A, double B, double mA, double mB, double S) {
  if (prod_le0(A, B)) return 0.0;
  const int ev = exp_of(maxF_nn(absF(A), absF(B)));
  const int em = exp_of(maxF_nn(mA, mB));
  const float a = f32_of(A, -ev), b = f32_of(B, -ev);
  const float ma = f32_of(mA, -em), mb = f32_of(mB, -em);
  const float w8 = (a * mb * mb + b * ma * ma) / (ma * mb * (ma + mb));
  const float g = fminf(fminf(fabsf(w8), fabsf(a) / ma), fabsf(b) / mb);
  return signF(f64_of(g, ev - em), S);
}
#endif

// The limited face flux of ale_kn_fluxelvl for the pair (i1, i2=i1+2),
// returning (fcflux(i1), fcflux(i2)) (ale_kn_advectors.f90:48-78).
__device__ __forceinline__ void elvl_pair(int iel, int i1, const int* nb, const int* fc,
                                          const d4* cnbasis, const double* own_b,
                                          double r1, double r2, const double* elvar,
                                          double rv, double& o1, double& o2) {
  const int i2 = i1 + 2;
  const int iel2 = nb[i2];
  int j2 = fc[i2];
  double r3 = own_b[i2] + own_b[(i2 + 1) & 3];
  double w5 = r3 + cget(cnbasis, iel2, j2) + cget(cnbasis, iel2, (j2 + 1) & 3);
  const int iel1 = nb[i1];
  j2 = fc[i1];
  double r4 = own_b[i1] + own_b[i1 + 1];
  double w6 = r4 + cget(cnbasis, iel1, j2) + cget(cnbasis, iel1, (j2 + 1) & 3);
  double w1 = rv - elvar[iel2];
  double w2 = elvar[iel1] - rv;
#if BL_MIXED
  const double grad = grad_f32(w1, w2, w5, w6, w2);
#else
  double w3 = absF(w1), w4 = absF(w2);
  double w8 = DIV(w1 * w6 * w6 + w2 * w5 * w5, w5 * w6 * (w5 + w6));
  double grad = sign_of(minF(minF(absF(w8), DIV(w3, w5)), DIV(w4, w6)), w2);
  if (prod_le0(w1, w2)) grad = 0.0;
#endif
  o1 = r1 * (rv + grad * (r3 - half(r1)));
  o2 = r2 * (rv - grad * (r4 - half(r2)));
  (void)iel;
}

// ================================================================ k_ale_flux

template <int BS, bool BATCH>
__global__ void __launch_bounds__(BS) k_ale_flux(DevFields F, DevCfg C) {
  const int iel = blockIdx.x * BS + threadIdx.x;
  if (iel >= F.nel) return;
  DevStep* S = el_step<BATCH>(F, iel);
  if (halted_a(S) || !ale_on(C, S)) return;
  const double dt = S->dt;
  const double zc = C.zerocut;
  const int4 nd = __ldg(F.ielnd + iel);
  const int n[4] = {nd.x, nd.y, nd.z, nd.w};
#if BL_FAST_ALGEBRA
  // Fast build: the face's swept volume from the face vector (Dx, Dy) and
  // the differences and sums of the mesh velocity -ubar at its ends: the
  // reference's quarter(a1*b3 - a3*b1) of the quad (x0(j), x0(j+1),
  // x1(j+1), x1(j)) with x1 = x0 - dt*ubar expands (exactly in real
  // arithmetic) to dt/4 * (2 (Dy Su - Dx Sv) + dt (Du Sv - Dv Su)), which
  // also avoids the cancellation of subtracting positions at two times.
  double x0[4], y0[4], ub[4], vb[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    x0[j] = F.ndx[n[j]];
    y0[j] = F.ndy[n[j]];
    ub[j] = F.ndubar[n[j]];
    vb[j] = F.ndvbar[n[j]];
  }
#else
  double x0[4], y0[4], x1[4], y1[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    x0[j] = F.ndx[n[j]];
    y0[j] = F.ndy[n[j]];
    // mesh velocity -ubar (zeul), x += dt*(-ubar)
    x1[j] = x0[j] + dt * (-F.ndubar[n[j]]);
    y1[j] = y0[j] + dt * (-F.ndvbar[n[j]]);
  }
#endif
  double fv[4], fvn[4];
#pragma unroll
  for (int jj = 0; jj < 4; jj++) {
    const int jp = (jj + 1) & 3;
#if BL_FAST_ALGEBRA
    const double Dx = x0[jp] - x0[jj], Dy = y0[jp] - y0[jj];
    const double Du = ub[jp] - ub[jj], Dv = vb[jp] - vb[jj];
    const double Su = ub[jp] + ub[jj], Sv = vb[jp] + vb[jj];
    const double A = Dy * Su - Dx * Sv, B = Du * Sv - Dv * Su;
    double d = quarter(dt * fma(dt, B, twice(A)));
#else
    double d = face_dv(x0[jj], x0[jp], y0[jj], y0[jp], x1[jp], x1[jj], y1[jp], y1[jj]);
#endif
    fv[jj] = gtF(zc, d) ? 0.0 : d;
    double dn = -d;   // the neighbour's volume of the same face
    fvn[jj] = gtF(zc, dn) ? 0.0 : dn;
  }
  const int4 ee = __ldg(F.ielel + iel);
  const int nb[4] = {ee.x, ee.y, ee.z, ee.w};
  const int fcp = __ldg(F.ielfc + iel);
  const int fc[4] = {fc_of(fcp, 0), fc_of(fcp, 1), fc_of(fcp, 2), fc_of(fcp, 3)};
  // ale_kn_sumflux(fcdv)
  double totv = 0.0;
#pragma unroll
  for (int i1 = 0; i1 < 2; i1++) {
    const int i2 = i1 + 2;
    double w1 = fvn[i1], w2 = fvn[i2];
    if (nb[i1] == iel) w1 = 0.0;
    if (nb[i2] == iel) w2 = 0.0;
    totv = totv - fv[i1] - fv[i2] + w1 + w2;
  }
  // ale_kn_fluxelvl(cnwt, fcdv, eldensity)
  const d4 cw = F.cnwt[iel];
  const double ob[4] = {cw.x, cw.y, cw.z, cw.w};
  const double rv = F.rho[iel];
  double fm[4];
  elvl_pair(iel, 0, nb, fc, F.cnwt, ob, fv[0], fv[2], F.rho, rv, fm[0], fm[2]);
  elvl_pair(iel, 1, nb, fc, F.cnwt, ob, fv[1], fv[3], F.rho, rv, fm[1], fm[3]);
  F.fcdm[iel] = make_d4(fm[0], fm[1], fm[2], fm[3]);
  F.fcdv[iel] = make_d4(fv[0], fv[1], fv[2], fv[3]);
  F.cutm_el[iel] = totv;  // carried to k_ale_el
}

// ================================================================ k_ale_el

template <int BS, bool BATCH>
__global__ void __launch_bounds__(BS) k_ale_el(DevFields F, DevCfg C) {
  const int iel = blockIdx.x * BS + threadIdx.x;
  if (iel >= F.nel) return;
  DevStep* S = el_step<BATCH>(F, iel);
  if (halted_a(S) || !ale_on(C, S)) return;
  const double zc = C.zerocut;
  const int4 ee = __ldg(F.ielel + iel);
  const int nb[4] = {ee.x, ee.y, ee.z, ee.w};
  const int fcp = __ldg(F.ielfc + iel);
  const int fc[4] = {fc_of(fcp, 0), fc_of(fcp, 1), fc_of(fcp, 2), fc_of(fcp, 3)};
  const d4 fm4 = F.fcdm[iel];
  const double fm[4] = {fm4.x, fm4.y, fm4.z, fm4.w};
  // ale_kn_sumflux(fcdm): neighbour's flux of the shared face
  double nfm[4];
  double totm = 0.0;
#pragma unroll
  for (int i1 = 0; i1 < 2; i1++) {
    const int i2 = i1 + 2;
    double w1 = cget(F.fcdm, nb[i1], fc[i1]);
    double w2 = cget(F.fcdm, nb[i2], fc[i2]);
    nfm[i1] = w1;
    nfm[i2] = w2;
    if (nb[i1] == iel) w1 = 0.0;
    if (nb[i2] == iel) w2 = 0.0;
    totm = totm - fm[i1] - fm[i2] + w1 + w2;
  }
  const double totv = F.cutm_el[iel];
  // ale_kn_updatebasisel
  const double vpr = F.vol[iel], mpr = F.mass[iel];
  const double v1 = vpr + totv;
  const double m1 = mpr + totm;
  F.vpr[iel] = vpr;
  F.mpr[iel] = mpr;
  F.vol[iel] = v1;
  F.mass[iel] = m1;
  F.rho[iel] = DIV(m1, v1);
  // ale_kn_fluxelvl(cnmass, fcdm, elenergy)
  const d4 cm = F.cnmass[iel];
  const double ob[4] = {cm.x, cm.y, cm.z, cm.w};
  const double ev = F.e[iel];
  double ef[4];
  elvl_pair(iel, 0, nb, fc, F.cnmass, ob, fm[0], fm[2], F.e, ev, ef[0], ef[2]);
  elvl_pair(iel, 1, nb, fc, F.cnmass, ob, fm[1], fm[3], F.e, ev, ef[1], ef[3]);
  F.eflux[iel] = make_d4(ef[0], ef[1], ef[2], ef[3]);
  // ale_kn_fluxbasisnd: corner mass-flux basis and corner mass flux
  double cndm[4], cnfl = 0.0;
#pragma unroll
  for (int i1 = 0; i1 < 2; i1++) {
    const int i2 = i1 + 2;
    double w3 = nfm[i1], w4 = nfm[i2];
    if (nb[i1] == iel) w3 = 0.0;
    if (nb[i2] == iel) w4 = 0.0;
    double w1 = w3 - fm[i1];
    double w2 = w4 - fm[i2];
    w3 = quarter(w1 - w2);
    cndm[i1] = w3;
    cndm[i2] = w3;
    w3 = quarter(w1 + w2);
    cnfl = cnfl + w3;
  }
  F.cnflux[iel] = make_d4(cnfl, cnfl, cnfl, cnfl);
  // ale_kn_fluxndvl for u and v (ale_kn_advectors.f90:83-153): corner flux
  // pairs (ilndl, ilndr, ii) in loop order (ilfcl, icn) = (1,1),(1,2),(2,1),(2,2)
  const int4 nd = __ldg(F.ielnd + iel);
  const int n[4] = {nd.x, nd.y, nd.z, nd.w};
  double cu[4], cv[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    cu[j] = F.ndu[n[j]];
    cv[j] = F.ndv[n[j]];
  }
  double fu[4] = {0.0, 0.0, 0.0, 0.0}, fv[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int ilfcl = 0; ilfcl < 2; ilfcl++) {
    const int ilfcr = ilfcl + 2;
    const int iell = nb[ilfcl], ielr = nb[ilfcr];
    const int ifcl = fc[ilfcl] + 1, ifcr = fc[ilfcr] + 1;   // 1-based as in the reference
#pragma unroll
    for (int icn = 1; icn <= 2; icn++) {
      const int ilndl = ilfcl + icn - 1;                     // 0-based corners
      const int ilndr = ((ilfcr + 1) - icn + 1) % 4;
      const int ii = ilfcl + 2 * (icn - 1);
      const double cdb = cndm[ii];
      double rdu = 0.0, rdv = 0.0;
#if BL_FAST_ALGEBRA
      // Fast build: the two branches (the corner's mass flux towards the
      // left neighbour, cdb > 0, or from the right one, cdb < 0) are one
      // computation with the corners and the neighbour swapped: near is the
      // corner of the pair the limiter is centred on, far the other one,
      // and the right branch's inner and outer differences are the left
      // form's negated (exactly), so a single branch-free path serves both
      // and a warp with fluxes of both signs runs it once.
      const bool lft = gtF(cdb, 0.0);
      if (lft || gtF(0.0, cdb)) {
        const int nbe = lft ? iell : ielr;
        const int lnl = lft ? (ifcl + icn) % 4 : (ifcr + icn - 2) % 4;
        const int lnr = lft ? (ifcl - icn + 1) % 4 : (((ifcr - icn - 1) % 4) + 4) % 4;
        const int nearc = lft ? ilndl : ilndr, farc = lft ? ilndr : ilndl;
        const int4 m = __ldg(F.ielnd + nbe);
        const int mm[4] = {m.x, m.y, m.z, m.w};
        const int nbn = mm[lft ? lnl : lnr];
        const double rd0 = ob[nearc] - half(absF(cdb));
        const double w5 = ob[ilndl] + ob[ilndr];
        const double w6 = cget(F.cnmass, nbe, lnl) + cget(F.cnmass, nbe, lnr);
        const double den = w5 * w6 * (w5 + w6);
#pragma unroll
        for (int q = 0; q < 2; q++) {
          const double* cvar = q == 0 ? cu : cv;
          const double* nvar = q == 0 ? F.ndu : F.ndv;
          const double rv = cvar[nearc];
          const double I = cvar[farc] - rv, O = rv - nvar[nbn];
#if BL_MIXED
          const double grad = grad_f32(I, O, w5, w6, I);
          (void)den;
#else
          const double w8 = DIV(I * w6 * w6 + O * w5 * w5, den);
          double grad = sign_of(minF(minF(absF(w8), DIV(absF(O), w6)), DIV(absF(I), w5)), I);
          if (prod_le0(O, I)) grad = 0.0;
#endif
          const double rd = cdb * (rv + grad * rd0);
          if (q == 0) rdu = rd; else rdv = rd;
        }
      }
#else
      if (gtF(cdb, 0.0)) {
        const int lnl = (ifcl + icn) % 4;
        const int lnr = (ifcl - icn + 1) % 4;
        const int4 m = __ldg(F.ielnd + iell);
        const int mm[4] = {m.x, m.y, m.z, m.w};
        double rd0 = ob[ilndl] - half(cdb);
        double w5 = ob[ilndl] + ob[ilndr];
        double w6 = cget(F.cnmass, iell, lnl) + cget(F.cnmass, iell, lnr);
        const double den = w5 * w6 * (w5 + w6);
#pragma unroll
        for (int q = 0; q < 2; q++) {
          const double* cvar = q == 0 ? cu : cv;
          const double* nvar = q == 0 ? F.ndu : F.ndv;
          double rv = cvar[ilndl];
          double w1 = rv - nvar[mm[lnl]];
          double w2 = cvar[ilndr] - rv;
          double w3 = absF(w1), w4 = absF(w2);
          double w8 = DIV(w2 * w6 * w6 + w1 * w5 * w5, den);
          double grad = sign_of(minF(minF(absF(w8), DIV(w3, w6)), DIV(w4, w5)), w2);
          if (prod_le0(w1, w2)) grad = 0.0;
          double rd = cdb * (rv + grad * rd0);
          if (q == 0) rdu = rd; else rdv = rd;
        }
      }
      if (gtF(0.0, cdb)) {
        const int lnl = (ifcr + icn - 2) % 4;
        const int lnr = (((ifcr - icn - 1) % 4) + 4) % 4;
        const int4 m = __ldg(F.ielnd + ielr);
        const int mm[4] = {m.x, m.y, m.z, m.w};
        double rd0 = ob[ilndr] + half(cdb);
        double w5 = ob[ilndl] + ob[ilndr];
        double w6 = cget(F.cnmass, ielr, lnl) + cget(F.cnmass, ielr, lnr);
        const double den = w5 * w6 * (w5 + w6);
#pragma unroll
        for (int q = 0; q < 2; q++) {
          const double* cvar = q == 0 ? cu : cv;
          const double* nvar = q == 0 ? F.ndu : F.ndv;
          double rv = cvar[ilndr];
          double w1 = rv - cvar[ilndl];
          double w2 = nvar[mm[lnr]] - rv;
          double w3 = absF(w1), w4 = absF(w2);
          double w8 = DIV(w1 * w6 * w6 + w2 * w5 * w5, den);
          double grad = -sign_of(minF(minF(absF(w8), DIV(w3, w5)), DIV(w4, w6)), w2);
          if (prod_le0(w1, w2)) grad = 0.0;
          double rd = cdb * (rv + grad * rd0);
          if (q == 0) rdu = rd; else rdv = rd;
        }
      }
#endif
      fu[ilndl] = fu[ilndl] - rdu;
      fu[ilndr] = fu[ilndr] + rdu;
      fv[ilndl] = fv[ilndl] - rdv;
      fv[ilndr] = fv[ilndr] + rdv;
    }
  }
  F.cnfu[iel] = make_d4(fu[0], fu[1], fu[2], fu[3]);
  F.cnfv[iel] = make_d4(fv[0], fv[1], fv[2], fv[3]);
  (void)zc;
}

// ================================================================ k_ale_nd

template <int BS, bool BATCH>
__global__ void __launch_bounds__(BS) k_ale_nd(DevFields F, DevCfg C) {
  const int ind = blockIdx.x * BS + threadIdx.x;
  if (ind >= F.nnd) return;
  const DevStep* S = nd_step<BATCH>(F, ind);
  if (halted_a(S) || !ale_on(C, S)) return;
  const double dt = S->dt;
  // calcbasisnd + massbasisnd in element-major (ielsort2) order
  double v0 = 0.0, m0 = 0.0;
  const int b = __ldg(F.ne_off + ind), e = __ldg(F.ne_off + ind + 1);
  for (int k = b; k < e; k++) {
    const int c = __ldg(F.ne_ent + k);
    const int iel = c >> 2, j = c & 3;
    v0 = v0 + quarter(F.vpr[iel]);
    m0 = m0 + cget(F.cnmass, iel, j);
  }
  double m1 = m0;
  double fu = 0.0, fv = 0.0;
  for (int k = b; k < e; k++) {
    const int c = __ldg(F.ne_ent + k);
    const int iel = c >> 2, j = c & 3;
    m1 = m1 + cget(F.cnflux, iel, j);
    fu = fu + cget(F.cnfu, iel, j);
    fv = fv + cget(F.cnfv, iel, j);
  }
  const double cutm = C.dencut * v0;
  const int t = __ldg(F.indtype + ind);
  // ale_kn_activend(-1) / (-2) with indstatus = 2 (zeul)
  const bool au = (t != -1) && (t != -3);
  const bool av = (t != -2) && (t != -3);
  double u = F.ndu[ind], v = F.ndv[ind];
  if (au && gtF(m1, cutm)) u = DIV(u * m0 + fu, m1);
  if (av && gtF(m1, cutm)) v = DIV(v * m0 + fv, m1);
  F.ndu[ind] = u;
  F.ndv[ind] = v;
  // Eulerian vertex: x + dt*(-ubar)
  F.ndx[ind] = F.ndx[ind] + dt * (-F.ndubar[ind]);
  F.ndy[ind] = F.ndy[ind] + dt * (-F.ndvbar[ind]);
}

// ================================================================ k_ale_update

template <int BS, bool BATCH>
__global__ void __launch_bounds__(BS) k_ale_update(DevFields F, DevCfg C) {
  const int iel = blockIdx.x * BS + threadIdx.x;
  if (iel >= F.nel) return;
  DevStep* S = el_step<BATCH>(F, iel);
  if (halted_a(S) || !ale_on(C, S)) return;
  const int4 ee = __ldg(F.ielel + iel);
  const int nb[4] = {ee.x, ee.y, ee.z, ee.w};
  const int fcp = __ldg(F.ielfc + iel);
  const int fc[4] = {fc_of(fcp, 0), fc_of(fcp, 1), fc_of(fcp, 2), fc_of(fcp, 3)};
  // ale_kn_updateel: sumflux(flux) then the mass-weighted energy
  const d4 f4 = F.eflux[iel];
  const double ef[4] = {f4.x, f4.y, f4.z, f4.w};
  double elf = 0.0;
#pragma unroll
  for (int i1 = 0; i1 < 2; i1++) {
    const int i2 = i1 + 2;
    double w1 = cget(F.eflux, nb[i1], fc[i1]);
    double w2 = cget(F.eflux, nb[i2], fc[i2]);
    if (nb[i1] == iel) w1 = 0.0;
    if (nb[i2] == iel) w2 = 0.0;
    elf = elf - ef[i1] - ef[i2] + w1 + w2;
  }
  const double m1 = F.mass[iel], mpr = F.mpr[iel];
  const double cut = F.vpr[iel] * C.dencut;
  double e = F.e[iel];
  if (gtF(m1, cut)) e = DIV(e * mpr + elf, m1);
  // new corner masses (ale_kn_massbasisnd)
  const d4 cm = F.cnmass[iel], cf = F.cnflux[iel];
  F.cnmass[iel] = make_d4(cm.x + cf.x, cm.y + cf.y, cm.z + cf.z, cm.w + cf.w);
  // ale_dr_hydroupdate: geometry at the remapped vertices, density, EoS
  const int4 nd = __ldg(F.ielnd + iel);
  const int n[4] = {nd.x, nd.y, nd.z, nd.w};
  double x[4], y[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    x[j] = F.ndx[n[j]];
    y[j] = F.ndy[n[j]];
  }
  Iso g = getiso(x, y);
  if (gtF(0.0, g.vol)) atomicMax(&S->negvol_ale, iel + 1 - el_base<BATCH>(F, iel));
  const double rho = DIV(m1, g.vol);
  double p, cs2;
  eos_pc(C, __ldg(F.ielmat + iel), rho, e, p, cs2);
  F.a1[iel] = g.a1;
  F.a2[iel] = g.a2;
  F.a3[iel] = g.a3;
  F.b1[iel] = g.b1;
  F.b2[iel] = g.b2;
  F.b3[iel] = g.b3;
  F.cnwt[iel] = make_d4(g.w0, g.w1, g.w2, g.w3);
  F.vol[iel] = g.vol;
  F.rho[iel] = rho;
  F.e[iel] = e;
  F.p[iel] = p;
  F.cs2[iel] = cs2;
  // components are not advected; the update still refreshes their
  // geometry, density and EoS (geometry_dr_volume.f90:66-79)
  const int imx = F.elmx ? F.elmx[iel] : -1;
  if (imx >= 0) {
    const int c0 = F.imxfcp[imx], nc = F.imxncp[imx];
    for (int k = 0; k < nc; k++) {
      const int icp = c0 + k;
      const double cpv = times4(g.a1 * g.b3 - g.a3 * g.b1) * F.frvol[icp];
      const double cpr = DIV(F.cpm[icp], cpv);
      double cpp, cpc;
      eos_pc(C, __ldg(F.icpmat + icp), cpr, F.cpe[icp], cpp, cpc);
      F.cpvol[icp] = cpv;
      F.cprho[icp] = cpr;
      F.cpp[icp] = cpp;
      F.cpcs2[icp] = cpc;
    }
  }
}

static constexpr int BS_A = 128;
static constexpr int BS_AN = 256;

template <bool BATCH>
void launch_ale_t(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  const int ge = (F.nel + BS_A - 1) / BS_A;
  k_ale_flux<BS_A, BATCH><<<ge, BS_A, 0, s>>>(F, C);
  k_ale_el<BS_A, BATCH><<<ge, BS_A, 0, s>>>(F, C);
  if constexpr (!BATCH) {
    k_ale_nd<BS_AN, false><<<(F.nnd + BS_AN - 1) / BS_AN, BS_AN, 0, s>>>(F, C);
  } else {
    // block size chosen by the batch's autotuner (128, 256 or 512)
    if (F.nd_block == 128) k_ale_nd<128, true><<<(F.nnd + 127) / 128, 128, 0, s>>>(F, C);
    else if (F.nd_block == 512) k_ale_nd<512, true><<<(F.nnd + 511) / 512, 512, 0, s>>>(F, C);
    else k_ale_nd<256, true><<<(F.nnd + 255) / 256, 256, 0, s>>>(F, C);
  }
  k_ale_update<BS_A, BATCH><<<ge, BS_A, 0, s>>>(F, C);
}
void launch_ale(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  launch_ale_t<false>(F, C, s);
}
void launch_ale_batch(const DevFields& F, const DevCfg& C, cudaStream_t s) {
  launch_ale_t<true>(F, C, s);
}

}  // namespace BL_NS
}  // namespace bl
