// bl_noalloc.cu -- bl_getdt_noalloc: the getdt step without any allocation.
//
// Some callers cannot call cudaMalloc: a host that hands out every byte of
// device memory from its own pool, where an allocation behind its back
// would fail or break its accounting.  For them this entry point runs
// bl_getdt's computation (edge viscosity, elcs2+elvisc, CFL and divergence
// limits, dt selection) on device arrays the caller passes, in the
// reference's own layout, without a bl_ctx.  It launches the library's own
// exact-form k_getdt (hydro_kernels.cuh, compiled here like the exact
// build, without FMA contraction), reading the caller's 1-based (NCORN,nel)
// connectivity through RefLayout below; its results equal bl_getdt's in
// BL_FP_EXACT mode bit for bit.
//
// The only device memory it needs beyond the caller's arrays -- the
// per-block (value,index) partials of the two scans, the step header with
// the last-block ticket, and the two per-region tables -- is the fixed
// file-scope array g_noalloc_scratch below (1.5 MiB plus a 2 KiB tail).
// Every GPU that loads the library holds that array until the process
// exits.
//
// Host code must not use g_noalloc_scratch's name as an address: on the
// host it names a stand-in, not device memory.  The device address is
// looked up once per device with cudaGetSymbolAddress, with that device
// current, the first time bl_getdt_noalloc runs on it; that first call
// therefore belongs before any stream capture.  All calls share the array:
// calls that overlap on the GPU race.  Each call uploads the step header
// (ticket zero) and the region tables before launching, so nothing a
// previous call left behind is read.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "../../include/bookleaf_gb300.h"

#define BL_NS na
#include "hydro_kernels.cuh"

namespace {

constexpr int kBS = 128;                              // k_getdt block: one element a thread
constexpr int kMaxBlocks = BL_NOALLOC_MAX_NEL / kBS;  // 65,536

// The caller's arrays in the reference's layout: ielnd, ielel, ielfc are
// (NCORN,nel) INTEGER blocks, 1-based; ielreg is 1-based; the corner
// outputs are (NCORN,nel) REAL(8) blocks with no alignment beyond 8 bytes.
struct RefLayout {
  static __device__ __forceinline__ int4 row(const void* p, int e) {
    const int* a = static_cast<const int*>(p) + 4 * (size_t)e;
    return make_int4(__ldg(a) - 1, __ldg(a + 1) - 1, __ldg(a + 2) - 1, __ldg(a + 3) - 1);
  }
  static __device__ __forceinline__ int4 nodes(const bl::DevFields& F, int e) {
    return row(F.ielnd, e);
  }
  static __device__ __forceinline__ int4 nbrs(const bl::DevFields& F, int e) {
    return row(F.ielel, e);
  }
  static __device__ __forceinline__ int faces(const bl::DevFields& F, int e) {
    const int4 f = row(F.ielfc, e);
    return (f.x & 0xff) | ((f.y & 0xff) << 8) | ((f.z & 0xff) << 16) | ((f.w & 0xff) << 24);
  }
  // regions outside 1..BL_MAXREG read region 1's settings
  static __device__ __forceinline__ int reg(const bl::DevFields& F, int e) {
    const int r = __ldg(F.ielreg + e) - 1;
    return (r < 0 || r >= BL_MAXREG) ? 0 : r;
  }
  static __device__ __forceinline__ void corners(bl::d4* p, int e, const double* q) {
    double* o = reinterpret_cast<double*>(p) + 4 * (size_t)e;
    o[0] = q[0];
    o[1] = q[1];
    o[2] = q[2];
    o[3] = q[3];
  }
};

// What each call uploads to the scratch tail: the step header and the
// zdtnotreg / zmidlength tables.
struct Upload {
  bl::DevStep step;
  int zdtnotreg[BL_MAXREG];
  int zmidlength[BL_MAXREG];
};

// [0, kOffI): two double partials per block; [kOffI, kOffU): two int
// partials per block; then the upload.
constexpr size_t kOffI = 2 * sizeof(double) * kMaxBlocks;
constexpr size_t kOffU = kOffI + 2 * sizeof(int) * kMaxBlocks;
constexpr size_t kScratchBytes = kOffU + 2048;
static_assert(sizeof(Upload) <= 2048, "upload record");
static_assert(kOffU % 256 == 0, "upload alignment");

}  // namespace

// The scratch array (file scope, one per device that loads the library).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

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
  if (A.elcs2_out == A.elcs2) {
    set_err(error, BL_FAILURE, BL_HALT_ALL,
            "ERROR: bl_getdt_noalloc: elcs2_out must not alias elcs2");
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
  Upload* dU = reinterpret_cast<Upload*>(scratch + kOffU);

  // the kernel's view of the caller's arrays (connectivity and corner
  // outputs are read and written through RefLayout, not as the library's
  // own vectors)
  bl::DevFields F;
  std::memset(&F, 0, sizeof F);
  F.nel = A.nel;
  F.nnd = A.nnd;
  F.ielnd = reinterpret_cast<const int4*>(A.ielnd);
  F.ielel = reinterpret_cast<const int4*>(A.ielel);
  F.ielfc = A.ielfc;
  F.ielreg = A.ielreg;
  F.indtype = A.indtype;
  F.ndx = const_cast<double*>(A.ndx);
  F.ndy = const_cast<double*>(A.ndy);
  F.ndu = const_cast<double*>(A.ndu);
  F.ndv = const_cast<double*>(A.ndv);
  F.rho = const_cast<double*>(A.eldensity);
  F.cs2 = const_cast<double*>(A.elcs2);
  F.cs2v = A.elcs2_out;
  F.vol = const_cast<double*>(A.elvolume);
  F.a1 = const_cast<double*>(A.a1);
  F.a3 = const_cast<double*>(A.a3);
  F.b1 = const_cast<double*>(A.b1);
  F.b3 = const_cast<double*>(A.b3);
  F.visc = A.elvisc;
  F.cnviscx = reinterpret_cast<bl::d4*>(A.cnviscx);
  F.cnviscy = reinterpret_cast<bl::d4*>(A.cnviscy);
  F.red_v = reinterpret_cast<double*>(scratch);
  F.red_i = reinterpret_cast<int*>(scratch + kOffI);
  F.step = &dU->step;
  bl::DevCfg C;
  std::memset(&C, 0, sizeof C);
  C.cvisc1 = config->cvisc1;
  C.cvisc2 = config->cvisc2;
  C.cfl_sf = config->cfl_sf;
  C.div_sf = config->div_sf;
  C.zcut = config->zcut;
  C.zerocut = config->zerocut;
  C.dt_g = config->dt_g;
  C.dt_min = config->dt_min;
  C.dt_max = config->dt_max;
  C.dt_initial = config->dt_initial;
  C.time_end = config->time_end;
  C.ztq = config->ztq;
  C.nreg = BL_MAXREG;
  C.zdtnotreg = dU->zdtnotreg;
  C.zmidlength = dU->zmidlength;

  Upload U;
  std::memset(&U, 0, sizeof U);
  U.step.time = ts->time;
  U.step.dt = ts->dt;
  U.step.dts = ts->dts;
  U.step.nstep = ts->nstep;
  U.step.idtel = ts->idtel;
  for (int i = 0; i < BL_MAXREG; i++) {
    U.zdtnotreg[i] = config->zdtnotreg[i] ? 1 : 0;
    U.zmidlength[i] = config->zmidlength[i] ? 1 : 0;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  r = cudaMemcpyAsync(dU, &U, sizeof U, cudaMemcpyHostToDevice, s);
  if (r != cudaSuccess) {
    set_err(error, BL_FAILURE, BL_HALT_ALL,
            "ERROR: bl_getdt_noalloc: uploading the step header failed");
    return BL_FAILURE;
  }
  const int blocks = (A.nel + kBS - 1) / kBS;
  bl::na::k_getdt<kBS, false, RefLayout><<<blocks, kBS, 0, s>>>(F, C);
  bl::DevStep R;
  r = cudaGetLastError();
  if (r == cudaSuccess)
    r = cudaMemcpyAsync(&R, &dU->step, sizeof R, cudaMemcpyDeviceToHost, s);
  if (r == cudaSuccess) r = cudaStreamSynchronize(s);
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
