// bl_noalloc.cu -- bl_getdt_noalloc: the getdt step without any allocation.
//
// Some callers cannot call cudaMalloc: a host that hands out every byte of
// device memory from its own pool, where an allocation behind its back
// would fail or break its accounting.  For them this entry point runs the computation
// of bl_getdt (k_getdt: edge viscosity, elcs2+elvisc, CFL and divergence
// limits, dt selection) on device arrays the caller passes, in the
// reference's own layout, without a bl_ctx.  The only device memory it
// needs beyond those arrays -- the per-block (value,index) partials of the
// two scans, the last-block ticket and the result record -- is the fixed
// file-scope array g_noalloc_scratch below (1.5 MiB plus a 256-byte tail).
// Every GPU that loads the library holds that array until the process exits.
//
// Host code must not use g_noalloc_scratch's name as an address: on the
// host it names a stand-in, not device memory.  The device address is
// looked up once per device with cudaGetSymbolAddress, with that device
// current, the first time bl_getdt_noalloc runs on it; that first call
// therefore belongs before any stream capture.  All calls share the array:
// calls that overlap on the GPU race, and each call clears the ticket and
// the result record it relies on before launching.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "../../include/bookleaf_gb300.h"

#define BL_NS na
#include "hydro_kernels.cuh"

namespace {

constexpr int kBS = 128;
constexpr int kMaxBlocks = BL_NOALLOC_MAX_NEL / kBS;  // 65,536

struct NaResult {
  double time, dt, cfl_rdt, div_rdt;
  int nstep, idtel, sdt, err_code;
  int cfl_idt, div_idt;
  unsigned int ticket;
  int pad;
};

// [0, 16*kMaxBlocks): two double partials per block; then two int
// partials per block; then the result record.
constexpr size_t kOffI = 2 * sizeof(double) * kMaxBlocks;
constexpr size_t kOffR = kOffI + 2 * sizeof(int) * kMaxBlocks;
constexpr size_t kScratchBytes = kOffR + 256;
static_assert(sizeof(NaResult) <= 256, "result record");

}  // namespace

// The scratch array (file scope, one per device that loads the library).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

struct NaParams {
  bl_getdt_arrays A;
  double cvisc1, cvisc2, zerocut, zcut, cfl_sf, div_sf, dt_g, dt_min, dt_max, dt_initial;
  double time, dt;
  int nstep, ztq, nreg, pad;
  unsigned char zdtnotreg[BL_MAXREG], zmidlength[BL_MAXREG];
};

using bl::maxF;
using bl::minF;
using bl::signF;
using bl::na::cfl_min;
using bl::na::div_max;
using bl::na::min_dlm;
using bl::na::min_dln;

// The body of k_getdt (hydro_kernels.cuh) on reference-layout arrays:
// hydro_kn_initeviscosity / limiteviscosity / geteviscosity
// (hydro_kn_edgeviscosity.f90:30-282), hydro_dr_getcs2, hydro_kn_getdtcfl /
// getdtdiv (hydro_kn_getdt.f90:30-122), time_dr_end (time_dr_advance.f90).
__global__ void __launch_bounds__(kBS) k_getdt_noalloc(NaParams P, unsigned char* scratch) {
  const bl_getdt_arrays& A = P.A;
  double* red_v = reinterpret_cast<double*>(scratch);
  int* red_i = reinterpret_cast<int*>(scratch + kOffI);
  NaResult* R = reinterpret_cast<NaResult*>(scratch + kOffR);
  const int iel = blockIdx.x * kBS + threadIdx.x;
  double cflv = HUGE_VAL;
  int cfli = 0x7fffffff;
  double divv = DBL_MIN;
  int divi = -1;
  if (iel < A.nel) {
    int n[4];
#pragma unroll
    for (int j = 0; j < 4; j++) n[j] = A.ielnd[4 * iel + j] - 1;
    double x[4], y[4], u[4], v[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      x[j] = A.ndx[n[j]];
      y[j] = A.ndy[n[j]];
      u[j] = A.ndu[n[j]];
      v[j] = A.ndv[n[j]];
    }
    const double zc = P.zerocut;
    const double rho0 = A.eldensity[iel];
    double visc = 0.0;
    if (!P.ztq) {
      double du[4], dv[4], dx[4], dy[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int jn = (j + 1) & 3;
        du[j] = u[jn] - u[j];
        dv[j] = v[jn] - v[j];
        dx[j] = x[jn] - x[j];
        dy[j] = y[jn] - y[j];
      }
      int nb[4], fc[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        nb[j] = A.ielel[4 * iel + j] - 1;
        fc[j] = A.ielfc[4 * iel + j] - 1;
      }
      double lu[4], lx[4], uh[4], vh[4], xh[4], yh[4];
      double sc[4][2];
      double edv[4];
#pragma unroll
      for (int s = 0; s < 2; s++) {
        const int in1 = nb[s], in2 = nb[s + 2];
        const int f1 = fc[s], f2 = fc[s + 2];
#pragma unroll
        for (int e2 = 0; e2 < 2; e2++) {
          const int is = e2 == 0 ? ((s + 3) & 3) : (s + 1);
          double w1 = du[is], w2 = dv[is], w3 = dx[is], w4 = dy[is];
          double den = sqrt(w1 * w1 + w2 * w2);
          lu[is] = den;
          den = 1.0 / maxF(den, zc);
          double uhat = w1 * den, vhat = w2 * den;
          den = sqrt(w3 * w3 + w4 * w4);
          lx[is] = den;
          den = 1.0 / maxF(den, zc);
          double xhat = w3 * den, yhat = w4 * den;
          uh[is] = uhat;
          vh[is] = vhat;
          xh[is] = xhat;
          yh[is] = yhat;
          den = w3 * xhat + w4 * yhat;
          w1 = (w1 * uhat + w2 * vhat) / signF(maxF(fabs(den), zc), den);
          w1 = 1.0 / signF(maxF(fabs(w1), zc), w1);
          const int ins1 = e2 == 0 ? ((f1 + 1) & 3) : ((f1 + 3) & 3);
          const int ins2 = e2 == 0 ? ((f2 + 3) & 3) : ((f2 + 1) & 3);
          double r1 = 0.0, r2 = 0.0;
          if (in1 != iel) {
            const int a = A.ielnd[4 * in1 + ins1] - 1, b = A.ielnd[4 * in1 + ((ins1 + 1) & 3)] - 1;
            double ddx = A.ndx[b] - A.ndx[a], ddy = A.ndy[b] - A.ndy[a];
            double ddu = A.ndu[b] - A.ndu[a], ddv = A.ndv[b] - A.ndv[a];
            double dn = ddx * xhat + ddy * yhat;
            double q = (ddu * uhat + ddv * vhat) / signF(maxF(fabs(dn), zc), dn);
            r1 = q * w1;
          }
          if (in2 != iel) {
            const int a = A.ielnd[4 * in2 + ins2] - 1, b = A.ielnd[4 * in2 + ((ins2 + 1) & 3)] - 1;
            double ddx = A.ndx[b] - A.ndx[a], ddy = A.ndy[b] - A.ndy[a];
            double ddu = A.ndu[b] - A.ndu[a], ddv = A.ndv[b] - A.ndv[a];
            double dn = ddx * xhat + ddy * yhat;
            double q = (ddu * uhat + ddv * vhat) / signF(maxF(fabs(dn), zc), dn);
            r2 = q * w1;
          }
          sc[is][0] = r1;
          sc[is][1] = r2;
        }
        const int is1 = (s + 3) & 3, is2 = s + 1;
        if (in1 == iel) {
          const double val = (A.indtype[n[s]] < 0 && A.indtype[n[(s + 1) & 3]] < 0 && in2 != iel) ? 1.0 : 0.0;
          sc[is1][0] = val;
          sc[is2][0] = val;
        }
        if (in2 == iel) {
          const double val = (A.indtype[n[s + 2]] < 0 && A.indtype[n[(s + 3) & 3]] < 0 && in1 != iel) ? 1.0 : 0.0;
          sc[is1][1] = val;
          sc[is2][1] = val;
        }
        const double cs2i = A.elcs2[iel];
#pragma unroll
        for (int e2 = 0; e2 < 2; e2++) {
          const int is = e2 == 0 ? is1 : is2;
          const int ins = nb[is];
          double w1 = P.cvisc1 * sqrt(0.5 * (cs2i + A.elcs2[ins]));
          double w2 = sc[is][0], w3 = sc[is][1];
          w2 = minF(minF(minF(0.5 * (w2 + w3), 2.0 * w2), 2.0 * w3), 1.0);
          w2 = maxF(0.0, w2);
          double w4 = lu[is];
          w3 = 0.5 * (1.0 - w2) * (rho0 + A.eldensity[ins]) * (w1 + P.cvisc2 * w4);
          edv[is] = w3;
          w4 = 2.0 * w4 / maxF(rho0, zc);
          visc = maxF(visc, w3 * w4);
        }
      }
      const double xc = 0.25 * (x[0] + x[1] + x[2] + x[3]);
      const double yc = 0.25 * (y[0] + y[1] + y[2] + y[3]);
      double edx[4], edy[4];
#pragma unroll
      for (int f = 0; f < 4; f++) {
        const int ins = (f + 1) & 3;
        double w3 = 0.5 * (x[f] + x[ins]);
        double w6 = 0.5 * (y[f] + y[ins]);
        double w7 = sqrt((xc - w3) * (xc - w3) + (yc - w6) * (yc - w6));
        double w8 = lx[f];
        double den = 1.0 / w7;
        double xhat = (yc - w6) * den, yhat = (w3 - xc) * den;
        double w33 = xhat * xh[f] + yhat * yh[f];
        den = -(signF(1.0, w33) * w7);
        xhat = xhat * den;
        yhat = yhat * den;
        double uhat = du[f], vhat = dv[f];
        double w5 = lu[f];
        double w6b = uhat * xhat + vhat * yhat;
        den = w6b / maxF(w5, zc);
        edx[f] = edv[f] * uhat * den;
        edy[f] = edv[f] * vhat * den;
        if ((w5 <= zc) || (w6b <= zc) || (w7 <= zc) || (w8 <= zc)) {
          edx[f] = 0.0;
          edy[f] = 0.0;
        }
      }
      A.cnviscx[4 * iel + 0] = edx[0] - edx[3];
      A.cnviscx[4 * iel + 1] = edx[1] - edx[0];
      A.cnviscx[4 * iel + 2] = edx[2] - edx[1];
      A.cnviscx[4 * iel + 3] = edx[3] - edx[2];
      A.cnviscy[4 * iel + 0] = edy[0] - edy[3];
      A.cnviscy[4 * iel + 1] = edy[1] - edy[0];
      A.cnviscy[4 * iel + 2] = edy[2] - edy[1];
      A.cnviscy[4 * iel + 3] = edy[3] - edy[2];
      A.elvisc[iel] = visc;
    } else {
      visc = A.elvisc[iel];
    }
    const double cs2v = A.elcs2[iel] + visc;
    A.elcs2_out[iel] = cs2v;
    int ireg = A.ielreg[iel] - 1;
    if (ireg < 0 || ireg >= BL_MAXREG) ireg = 0;  // out-of-range regions read region 1
    double r11;
    if (P.zdtnotreg[ireg]) {
      r11 = DBL_MAX;
    } else {
      double w1 = P.zmidlength[ireg] ? min_dlm(x, y) : min_dln(x, y, P.zcut);
      r11 = w1 / cs2v;
    }
    cflv = r11;
    cfli = iel;
    const double A1 = A.a1[iel], A3 = A.a3[iel], B1 = A.b1[iel], B3 = A.b3[iel];
    double w1 = u[0] * (-B3 + B1) + v[0] * (A3 - A1) + u[1] * (B3 + B1) + v[1] * (-A3 - A1) +
                u[2] * (B3 - B1) + v[2] * (-A3 + A1) + u[3] * (-B3 - B1) + v[3] * (A3 + A1);
    w1 = fabs(w1) / A.elvolume[iel];
    if (w1 > divv) {
      divv = w1;
      divi = iel;
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
  __shared__ double s_cv[kBS / 32], s_dv[kBS / 32];
  __shared__ int s_ci[kBS / 32], s_di[kBS / 32];
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
    for (int w = 1; w < kBS / 32; w++) {
      cfl_min(cflv, cfli, s_cv[w], s_ci[w]);
      div_max(divv, divi, s_dv[w], s_di[w]);
    }
    red_v[2 * blockIdx.x] = cflv;
    red_i[2 * blockIdx.x] = cfli;
    red_v[2 * blockIdx.x + 1] = divv;
    red_i[2 * blockIdx.x + 1] = divi;
    __threadfence();
    unsigned int t = atomicAdd(&R->ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  cflv = HUGE_VAL;
  cfli = 0x7fffffff;
  divv = DBL_MIN;
  divi = -1;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kBS) {
    cfl_min(cflv, cfli, ((volatile double*)red_v)[2 * b], ((volatile int*)red_i)[2 * b]);
    div_max(divv, divi, ((volatile double*)red_v)[2 * b + 1], ((volatile int*)red_i)[2 * b + 1]);
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
  for (int w = 1; w < kBS / 32; w++) {
    cfl_min(cflv, cfli, s_cv[w], s_ci[w]);
    div_max(divv, divi, s_dv[w], s_di[w]);
  }
  R->ticket = 0;
  if (cflv < 0.0) {
    R->err_code = 1;
    return;
  }
  const double rdt_cfl = P.cfl_sf * sqrt(cflv);
  const double rdt_div = P.div_sf / divv;
  R->cfl_rdt = rdt_cfl;
  R->cfl_idt = cfli + 1;
  R->div_rdt = rdt_div;
  R->div_idt = divi + 1;
  double mind = P.dt_max;
  int mini = -1, mins = 0;
  double g = P.dt_g * P.dt;
  if (g < mind) { mind = g; mini = -1; mins = 1; }
  if (P.nstep == 0 && P.dt_initial < mind) { mind = P.dt_initial; mini = -1; mins = 2; }
  if (rdt_cfl < mind) { mind = rdt_cfl; mini = cfli + 1; mins = 3; }
  if (rdt_div < mind) { mind = rdt_div; mini = divi + 1; mins = 4; }
  R->nstep = P.nstep + 1;
  R->dt = mind;
  R->sdt = mins;
  R->idtel = mini;
  R->time = P.time + mind;
  R->err_code = (mind < P.dt_min) ? 2 : 0;
}

// Device address of g_noalloc_scratch per device ordinal, looked up once.
constexpr int kMaxDevices = 64;
unsigned char* g_scratch_addr[kMaxDevices] = {};

void set_err(bl_error* e, int ierr, int iout, const char* msg) {
  if (!e) return;
  e->ierr = ierr;
  e->iout = iout;
  std::strncpy(e->serr, msg ? msg : "", BL_SLEN);
  e->serr[BL_SLEN] = 0;
}

const char* kSdtNames[5] = {" MAXIMUM", "  GROWTH", " INITIAL", "     CFL", "     DIV"};

}  // namespace

extern "C" int bl_getdt_noalloc(const bl_getdt_arrays* arrays, const bl_config* config,
                                bl_timestep* ts, void* stream, bl_error* error) {
  set_err(error, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (!arrays || !config || !ts) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_getdt_noalloc: null argument");
    return BL_FAILURE;
  }
  const bl_getdt_arrays& A = *arrays;
  if (A.nel < 1 || A.nnd < 4) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_getdt_noalloc: empty mesh");
    return BL_FAILURE;
  }
  if (A.nel > BL_NOALLOC_MAX_NEL) {
    set_err(error, BL_FAILURE, BL_HALT_ALL,
            "ERROR: bl_getdt_noalloc: nel exceeds BL_NOALLOC_MAX_NEL (8,388,608)");
    return BL_FAILURE;
  }
  if (!A.ndx || !A.ndy || !A.ndu || !A.ndv || !A.indtype || !A.ielnd || !A.ielel || !A.ielfc ||
      !A.ielreg || !A.eldensity || !A.elcs2 || !A.a1 || !A.a3 || !A.b1 || !A.b3 ||
      !A.elvolume || !A.cnviscx || !A.cnviscy || !A.elvisc || !A.elcs2_out) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_getdt_noalloc: null array");
    return BL_FAILURE;
  }
  int dev = 0;
  cudaError_t r = cudaGetDevice(&dev);
  if (r != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_getdt_noalloc: no usable CUDA device");
    return BL_FAILURE;
  }
  if (!g_scratch_addr[dev]) {
    // set-up, once per device, with that device current
    void* p = nullptr;
    r = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (r != cudaSuccess || !p) {
      set_err(error, BL_FAILURE, BL_HALT_ALL,
              "ERROR: bl_getdt_noalloc: cudaGetSymbolAddress of the scratch array failed");
      return BL_FAILURE;
    }
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  unsigned char* scratch = g_scratch_addr[dev];
  NaParams P;
  std::memset(&P, 0, sizeof P);
  P.A = A;
  P.cvisc1 = config->cvisc1;
  P.cvisc2 = config->cvisc2;
  P.zerocut = config->zerocut;
  P.zcut = config->zcut;
  P.cfl_sf = config->cfl_sf;
  P.div_sf = config->div_sf;
  P.dt_g = config->dt_g;
  P.dt_min = config->dt_min;
  P.dt_max = config->dt_max;
  P.dt_initial = config->dt_initial;
  P.time = ts->time;
  P.dt = ts->dt;
  P.nstep = ts->nstep;
  P.ztq = config->ztq;
  for (int i = 0; i < BL_MAXREG; i++) {
    P.zdtnotreg[i] = config->zdtnotreg[i] ? 1 : 0;
    P.zmidlength[i] = config->zmidlength[i] ? 1 : 0;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the ticket and the result record must start from zero on every call
  r = cudaMemsetAsync(scratch + kOffR, 0, sizeof(NaResult), s);
  if (r != cudaSuccess) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_getdt_noalloc: clearing scratch failed");
    return BL_FAILURE;
  }
  const int blocks = (A.nel + kBS - 1) / kBS;
  k_getdt_noalloc<<<blocks, kBS, 0, s>>>(P, scratch);
  NaResult R;
  r = cudaMemcpyAsync(&R, scratch + kOffR, sizeof R, cudaMemcpyDeviceToHost, s);
  if (r == cudaSuccess) r = cudaStreamSynchronize(s);
  if (r == cudaSuccess) r = cudaGetLastError();
  if (r != cudaSuccess) {
    char msg[BL_SLEN + 1];
    std::snprintf(msg, sizeof msg, "ERROR: CUDA %s in bl_getdt_noalloc", cudaGetErrorString(r));
    set_err(error, BL_FAILURE, BL_HALT_ALL, msg);
    return BL_FAILURE;
  }
  if (R.err_code == 1) {
    set_err(error, BL_FAILURE, BL_HALT_SINGLE, "ERROR: negative CFL condition in hydro_dr_getdt");
    return BL_FAILURE;
  }
  ts->nstep = R.nstep;
  ts->dt = R.dt;
  ts->time = R.time;
  ts->idtel = R.idtel;
  std::memset(ts->sdt, 0, sizeof ts->sdt);
  std::memcpy(ts->sdt, kSdtNames[R.sdt < 0 || R.sdt > 4 ? 0 : R.sdt], 8);
  // material names live with the caller; mdt is left for it to fill
  ts->imdt = -1;
  std::memset(ts->mdt, 0, sizeof ts->mdt);
  if (R.err_code == 2) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: dt < dt_min");
    return BL_FAILURE;
  }
  return BL_SUCCESS;
}
