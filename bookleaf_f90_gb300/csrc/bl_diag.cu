// bl_diag.cu -- the reference's run-time diagnostics on the device, so that a
// host printing them needs a few hundred bytes instead of the whole state:
//
//   bl_shortprint   hydro_dr_shortprint (hydro_dr_print.f90:49-170):
//                   hydro_kn_calc_shortprint per region or material over the
//                   elements and, for materials, the mixed-cell components
//                   (hydro_kn_print.F90:52-101), then
//                   hydro_kn_average_shortprint (:219-240)
//   bl_check_sod    check_dr_sod / check_kn_sod (check_dr_tests.f90:34-71,
//                   check_kn_tests.f90:33-111)
//
// Every sum is a fixed tree: each block owns a fixed range of elements, a
// block reduces in shared memory in a fixed order, and one thread adds the
// block partials in block order, so results are reproducible run to run.
// They differ from the reference's serial sums only in rounding.
#include <cfloat>
#include <cstring>

#include "bl_ctx.h"

namespace {

constexpr int kBS = 256;
constexpr int kItems = 8;            // elements per thread
constexpr int kSP = 9;               // vol, mass, ie, ke, pre, pmn, pmx, dmn, dmx

// block reduction of v (sum, min or max) into thread 0's return value
template <int OP>
__device__ double block_reduce(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = kBS / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      const double a = sh[threadIdx.x], b = sh[threadIdx.x + s];
      sh[threadIdx.x] = OP == 0 ? a + b : (OP == 1 ? (b < a ? b : a) : (b > a ? b : a));
    }
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// one flag's contribution of a thread's items (elements or components)
struct SPAcc {
  double vol = 0, mass = 0, ie = 0, ke = 0, pre = 0;
  double pmn = DBL_MAX, pmx = -DBL_MAX, dmn = DBL_MAX, dmx = -DBL_MAX;
  __device__ void add(double dencut, double vol_i, double m, double e, double p, double rho,
                      const bl::d4& wt, const double* u, const double* v) {
    const double c1 = dencut * vol_i;
    vol = vol + vol_i;
    if (m > c1) {
      mass = mass + m;
      ie = ie + e * m;
      pre = pre + m * p;
      if (p > pmx) pmx = p;
      if (p < pmn) pmn = p;
      if (rho > dmx) dmx = rho;
      if (rho < dmn) dmn = rho;
      const double w[4] = {wt.x, wt.y, wt.z, wt.w};
#pragma unroll
      for (int ic = 0; ic < 4; ic++) ke = 0.5 * w[ic] * rho * (u[ic] * u[ic] + v[ic] * v[ic]) + ke;
    }
  }
};

__device__ void write_partials(const SPAcc& a, double* sh, double* out) {
  const double s0 = block_reduce<0>(a.vol, sh);
  const double s1 = block_reduce<0>(a.mass, sh);
  const double s2 = block_reduce<0>(a.ie, sh);
  const double s3 = block_reduce<0>(a.ke, sh);
  const double s4 = block_reduce<0>(a.pre, sh);
  const double s5 = block_reduce<1>(a.pmn, sh);
  const double s6 = block_reduce<2>(a.pmx, sh);
  const double s7 = block_reduce<1>(a.dmn, sh);
  const double s8 = block_reduce<2>(a.dmx, sh);
  if (threadIdx.x == 0) {
    out[0] = s0; out[1] = s1; out[2] = s2; out[3] = s3; out[4] = s4;
    out[5] = s5; out[6] = s6; out[7] = s7; out[8] = s8;
  }
}

// element pass: part[(block * nflag + f) * kSP + q]
__global__ void __launch_bounds__(kBS) k_sp_elements(bl::DevFields F, int by_material, int nflag,
                                                     double dencut, double* part) {
  __shared__ double sh[kBS];
  const int base = blockIdx.x * kBS * kItems + threadIdx.x;
  for (int f = 1; f <= nflag; f++) {
    SPAcc a;
    for (int k = 0; k < kItems; k++) {
      const int i = base + k * kBS;
      if (i >= F.nel) break;
      const int flag = by_material ? F.ielmat[i] : F.ielreg[i] + 1;
      if (flag != f) continue;
      const int4 nd = F.ielnd[i];
      const double u[4] = {F.ndu[nd.x], F.ndu[nd.y], F.ndu[nd.z], F.ndu[nd.w]};
      const double v[4] = {F.ndv[nd.x], F.ndv[nd.y], F.ndv[nd.z], F.ndv[nd.w]};
      a.add(dencut, F.vol[i], F.mass[i], F.e[i], F.p[i], F.rho[i], F.cnwt[i], u, v);
    }
    write_partials(a, sh, part + ((size_t)blockIdx.x * nflag + (f - 1)) * kSP);
  }
}

// component pass (materials only): mixed cell m's components with the
// element's corner weights and velocities (utils_kn_mxgathercncp)
__global__ void __launch_bounds__(kBS) k_sp_components(bl::DevFields F, int nflag, double dencut,
                                                       double* part) {
  __shared__ double sh[kBS];
  const int base = blockIdx.x * kBS * kItems + threadIdx.x;
  for (int f = 1; f <= nflag; f++) {
    SPAcc a;
    for (int k = 0; k < kItems; k++) {
      const int m = base + k * kBS;
      if (m >= F.nmx) break;
      const int iel = F.imxel[m], c0 = F.imxfcp[m], nc = F.imxncp[m];
      const int4 nd = F.ielnd[iel];
      const double u[4] = {F.ndu[nd.x], F.ndu[nd.y], F.ndu[nd.z], F.ndu[nd.w]};
      const double v[4] = {F.ndv[nd.x], F.ndv[nd.y], F.ndv[nd.z], F.ndv[nd.w]};
      for (int c = c0; c < c0 + nc; c++) {
        if (F.icpmat[c] != f) continue;
        a.add(dencut, F.cpvol[c], F.cpm[c], F.cpe[c], F.cpp[c], F.cprho[c], F.cnwt[iel], u, v);
      }
    }
    write_partials(a, sh, part + ((size_t)blockIdx.x * nflag + (f - 1)) * kSP);
  }
}

// partials in block order, elements then components, then the averages
__global__ void k_sp_final(const double* pe, int nbe, const double* pc, int nbc, int nflag,
                           double dencut, double* out) {
  for (int f = threadIdx.x; f < nflag; f += blockDim.x) {
    double vol = 0, mass = 0, ie = 0, ke = 0, pre = 0;
    double pmn = DBL_MAX, pmx = -DBL_MAX, dmn = DBL_MAX, dmx = -DBL_MAX;
    for (int pass = 0; pass < 2; pass++) {
      const double* p = pass == 0 ? pe : pc;
      const int nb = pass == 0 ? nbe : nbc;
      for (int b = 0; b < nb; b++) {
        const double* q = p + ((size_t)b * nflag + f) * kSP;
        vol = vol + q[0];
        mass = mass + q[1];
        ie = ie + q[2];
        ke = ke + q[3];
        pre = pre + q[4];
        if (q[5] < pmn) pmn = q[5];
        if (q[6] > pmx) pmx = q[6];
        if (q[7] < dmn) dmn = q[7];
        if (q[8] > dmx) dmx = q[8];
      }
    }
    // hydro_kn_average_shortprint
    const double density = vol > 0.0 ? mass / vol : 0.0;
    const double pressure = mass > dencut * vol ? pre / mass : pre;
    double* o = out + (size_t)f * BL_SP_NQ;
    o[0] = vol; o[1] = mass; o[2] = ie; o[3] = ke; o[4] = pressure;
    o[5] = pmn; o[6] = pmx; o[7] = density; o[8] = dmn; o[9] = dmx;
  }
}

// sod (check_kn_tests.f90:64-111): exact density and energy at x relative
// to the interface at time t (gamma 1.4, the check's states)
__device__ void sod_exact(double xx, double time, double& rho, double& e) {
  rho = -DBL_MAX;
  e = -DBL_MAX;
  const double coeff = sqrt(1.4);
  if (xx <= -coeff * time) {
    rho = 1.0;
    e = 2.5;
  } else if (xx <= -0.07027281256118326961 * time) {
    const double ss = xx / time;
    const double velocity = (5.0 / 6.0) * (ss + coeff);
    const double tt = ((velocity - ss) * (velocity - ss)) / 1.4;
    rho = pow(tt, 2.5);
    e = rho * tt / (0.4 * rho);
  } else if (xx <= 0.92745262004894994908 * time) {
    rho = 0.42631942817849519385;
    e = 1.77760006942335264781;
  } else if (time <= 28.53627624872492075028) {
    if (xx <= 1.75215573203017816370 * time) {
      rho = 0.26557371170530706471;
      e = 2.85354088799095973738;
    } else {
      rho = 0.125;
      e = 2.0;
    }
  } else if (time < 40.68191725689148697880) {
    if (xx <= (50.0 - (time - 28.53627624872492075028) * 1.01019363599101820444)) {
      rho = 0.26557371170530706471;
      e = 2.85354088799095973738;
    } else {
      rho = 0.50939531774381657731;
      e = 3.82996297061558546292;
    }
  }
}

__global__ void __launch_bounds__(kBS) k_sod(bl::DevFields F, double time, double* part) {
  __shared__ double sh[kBS];
  const int base = blockIdx.x * kBS * kItems + threadIdx.x;
  double basis = 0.0, l1d = 0.0, l1e = 0.0;
  for (int k = 0; k < kItems; k++) {
    const int i = base + k * kBS;
    if (i >= F.nel) break;
    const int4 nd = F.ielnd[i];
    const double xx[4] = {F.ndx[nd.x], F.ndx[nd.y], F.ndx[nd.z], F.ndx[nd.w]};
    const double yy[4] = {F.ndy[nd.x], F.ndy[nd.y], F.ndy[nd.z], F.ndy[nd.w]};
    // geometry_kn_getcentroid (geometry_kn_centroid.f90:29-55)
    double cx = 0.0, rvol = 0.0;
#pragma unroll
    for (int i1 = 0; i1 < 4; i1++) {
      const int i2 = (i1 + 1) & 3;
      const double rr = xx[i1] * yy[i2] - xx[i2] * yy[i1];
      rvol = rvol + rr;
      cx = cx + rr * (xx[i1] + xx[i2]);
    }
    rvol = 0.5 * rvol;
    cx = rvol > 0.0 ? cx / (6.0 * rvol) : 0.0;
    double sr, se;
    sod_exact(cx - 50.0, time, sr, se);
    const double vol = F.vol[i];
    basis = basis + vol;
    l1d = fabs(F.rho[i] - sr) * vol + l1d;
    l1e = fabs(F.e[i] - se) * vol + l1e;
  }
  const double s0 = block_reduce<0>(basis, sh);
  const double s1 = block_reduce<0>(l1d, sh);
  const double s2 = block_reduce<0>(l1e, sh);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = s0;
    part[3 * blockIdx.x + 1] = s1;
    part[3 * blockIdx.x + 2] = s2;
  }
}

__global__ void k_sod_final(const double* part, int nb, double* out) {
  if (threadIdx.x != 0) return;
  double b = 0, d = 0, e = 0;
  for (int k = 0; k < nb; k++) {
    b = b + part[3 * k];
    d = d + part[3 * k + 1];
    e = e + part[3 * k + 2];
  }
  out[0] = d / b;
  out[1] = e / b;
}

int blocks_for(int n) { return n <= 0 ? 0 : (n + kBS * kItems - 1) / (kBS * kItems); }

void set_error(bl_error* e, int ierr, const char* msg) {
  if (!e) return;
  e->ierr = ierr;
  e->iout = BL_HALT_SINGLE;
  std::strncpy(e->serr, msg, BL_SLEN);
  e->serr[BL_SLEN] = 0;
}

// scratch of the diagnostics, grown on demand and kept with the context
double* scratch(bl_ctx* x, size_t n) {
  if (n <= x->diag_cap) return x->diag;
  if (x->diag) cudaFree(x->diag);
  x->diag = nullptr;
  x->diag_cap = 0;
  if (cudaMalloc(&x->diag, n * sizeof(double)) != cudaSuccess) return nullptr;
  x->diag_cap = n;
  return x->diag;
}

}  // namespace

extern "C" int bl_shortprint(bl_ctx* x, int table, double* out, int nflag, bl_error* e) {
  set_error(e, BL_SUCCESS, "");
  if (!x || !out || (table != 0 && table != 1) || x->ninst > 0) {
    set_error(e, BL_FAILURE, "ERROR: bl_shortprint: bad argument (or a batch context)");
    return BL_FAILURE;
  }
  const int nf = table == 1 ? x->s.nmat : x->s.nreg;
  if (nflag < nf) {
    set_error(e, BL_FAILURE, "ERROR: bl_shortprint: output holds fewer rows than flags");
    return BL_FAILURE;
  }
  const int nbe = blocks_for(x->s.nel);
  const int nbc = table == 1 && x->s.nmx > 0 ? blocks_for(x->s.nmx) : 0;
  double* d = scratch(x, (size_t)(nbe + nbc) * nf * kSP + (size_t)nf * BL_SP_NQ);
  if (!d) {
    set_error(e, BL_FAILURE, "ERROR: bl_shortprint: device allocation failed");
    return BL_FAILURE;
  }
  double* pe = d;
  double* pc = d + (size_t)nbe * nf * kSP;
  double* res = pc + (size_t)nbc * nf * kSP;
  const double dencut = x->c.dencut;
  if (nbe) k_sp_elements<<<nbe, kBS, 0, x->stream>>>(x->F, table, nf, dencut, pe);
  if (nbc) k_sp_components<<<nbc, kBS, 0, x->stream>>>(x->F, nf, dencut, pc);
  k_sp_final<<<1, 128, 0, x->stream>>>(pe, nbe, pc, nbc, nf, dencut, res);
  x->launches += (nbe ? 1 : 0) + (nbc ? 1 : 0) + 1;
  cudaError_t r = cudaMemcpyAsync(out, res, sizeof(double) * nf * BL_SP_NQ,
                                  cudaMemcpyDeviceToHost, x->stream);
  if (r == cudaSuccess) r = cudaStreamSynchronize(x->stream);
  if (r == cudaSuccess) r = cudaGetLastError();
  if (r != cudaSuccess) {
    set_error(e, BL_FAILURE, cudaGetErrorString(r));
    return BL_FAILURE;
  }
  return BL_SUCCESS;
}

extern "C" int bl_check_sod(bl_ctx* x, double time, double* l1_density, double* l1_energy,
                            bl_error* e) {
  set_error(e, BL_SUCCESS, "");
  if (!x || !l1_density || !l1_energy || x->ninst > 0) {
    set_error(e, BL_FAILURE, "ERROR: bl_check_sod: bad argument (or a batch context)");
    return BL_FAILURE;
  }
  const int nb = blocks_for(x->s.nel);
  double* d = scratch(x, (size_t)3 * nb + 2);
  if (!d) {
    set_error(e, BL_FAILURE, "ERROR: bl_check_sod: device allocation failed");
    return BL_FAILURE;
  }
  k_sod<<<nb, kBS, 0, x->stream>>>(x->F, time, d);
  k_sod_final<<<1, 32, 0, x->stream>>>(d, nb, d + 3 * nb);
  x->launches += 2;
  double h[2];
  cudaError_t r = cudaMemcpyAsync(h, d + 3 * nb, sizeof h, cudaMemcpyDeviceToHost, x->stream);
  if (r == cudaSuccess) r = cudaStreamSynchronize(x->stream);
  if (r == cudaSuccess) r = cudaGetLastError();
  if (r != cudaSuccess) {
    set_error(e, BL_FAILURE, cudaGetErrorString(r));
    return BL_FAILURE;
  }
  *l1_density = h[0];
  *l1_energy = h[1];
  return BL_SUCCESS;
}
