// bl_device.cuh -- device-side data structures and helpers shared by the
// hydro (Lagrangian) and ALE kernels.
//
// Layout in HBM (one partition, structure of arrays):
//   node fields     double[nnd]            ndx, ndy, ndu, ndv, ndubar, ...
//   element fields  double[nel]            eldensity, elenergy, ...
//   corner fields   d4[nel]           cnwt, cnmass, cnviscx, ... (the
//                                          reference's (NCORN,nel) block: the
//                                          4 corners of one element are one
//                                          32-byte vector load)
//   connectivity    int4[nel] (0-based)    ielnd, ielel; ielfc packed as four
//                                          bytes in one int
//   node->corner    CSR (offsets, entries) in the summation order of the
//                   reference's scatter loops, so node sums are computed by
//                   gathers without atomics and are deterministic.
#pragma once
#include "bl_fp64.cuh"
#include <cstdint>
#include <cuda_runtime.h>

namespace bl {

// 32-byte aligned vector of the four corner (or face) values of one element.
using d4 = double4_32a;
__host__ __device__ __forceinline__ d4 make_d4(double x, double y, double z, double w) {
  return make_double4_32a(x, y, z, w);
}

// Runtime state of the time loop that lives on the device.  The host reads
// it back once per bl_getdt call; bl_run never reads it inside the loop.
struct DevStep {
  double time, dt, dts;
  double rdt;           // 1/dt (hourglass filter), set with dt
  double cfl_rdt, div_rdt;
  int nstep, idtel, sdt, imdt;
  int cfl_idt, div_idt;
  int ierr, iout;       // error_t of the first failure
  int err_code;         // 0 none, 1 negative CFL, 2 dt<dt_min, 3 neg volume
  int negvol_pred;      // 1 + last element with V<0 in the predictor (0: none)
  int negvol_corr;      // same for the corrector
  int negvol_ale;       // same for the ALE update
  int run_mode;         // 1 inside bl_run: kernels stop after time_end/error
  int stop_next;        // set by getdt when time >= time_end (bl_run)
  int halted;           // kernels return at once when set
  int nrecord;          // steps recorded in the history buffer
  unsigned int ticket;  // last-block counter of the dt reduction
  int pad;
};

// Per-mesh controls of a batch (independent meshes advanced together, each
// with its own dt and time): the time-step parameters of its control file,
// its element range and the k_getdt blocks that cover it.
struct DevInst {
  double dt_g, dt_min, dt_max, dt_initial, time_end;
  int el_begin, el_end;
  int blk_begin, blk_end;
};

struct StepRec {        // mirrors bl_step_record
  double time, dt;
  int nstep, idtel, sdt_code, ierr;
};

// Configuration scalars and the small per-region / per-material tables.
struct DevCfg {
  double cvisc1, cvisc2, cfl_sf, div_sf;
  double zcut, zerocut, dencut, accut, ccut, pcut;
  double dt_g, dt_min, dt_max, dt_initial, time_end;
  double ale_mintime, ale_maxtime;
  int ztq, zhg, zsp, nreg, nmat, ale_zexist, ale_zeul, adv_type;
  int max_records, pad0;
  const double* kappareg;    // [nreg]
  const double* pmeritreg;   // [nreg]
  const int* zdtnotreg;      // [nreg]
  const int* zmidlength;     // [nreg]
  const int* eos_type;       // [nmat+1]
  const double* eos_param;   // [(nmat+1)*6]
  const double* eos_gm1;     // [nmat+1]  param1-1           (ideal gas)
  const double* eos_ggm1;    // [nmat+1]  param1*(param1-1)  (ideal gas)
};

struct DevFields {
  int nel, nnd, ncp, nmx;
  // connectivity (0-based)
  const int4* ielnd;
  const int4* ielel;
  const int* ielfc;          // 4 x 8-bit face numbers 0..3
  const int* ielreg;         // 0-based region
  const int* ielmat;         // material (<=0: mixed / void)
  const int* indtype;
  const int* elmx;           // mixed-cell index of an element (-1: pure)
  // node -> corner CSR, corner-major order (hydro_kn_scatteracceleration)
  const int* nc_off;         // [nnd+1]
  const int* nc_ent;         // entries 4*iel+corner
  // node -> corner CSR, element-major order (ALE nodal sums)
  const int* ne_off;
  const int* ne_ent;
  // node fields
  double *ndx, *ndy, *ndu, *ndv, *ndubar, *ndvbar, *ndxn, *ndyn;
  // element fields
  double *rho, *e, *p, *cs2, *cs2v, *vol, *mass, *visc;
  double *a1, *a2, *a3, *b1, *b2, *b3;
  double *rho_h;             // half-step density (predictor -> node kernel)
  double* e_scr;             // elenergy0 / ALE scratch
  // corner fields
  d4 *cnwt, *cnmass, *cnviscx, *cnviscy, *cnfx, *cnfy, *spmass;
  d4* cnwt_h;           // half-step corner volumes
  // mixed cells (flattened; components of one cell contiguous)
  const int* imxel;          // 0-based element of a mixed cell
  const int* imxfcp;         // 0-based first component
  const int* imxncp;
  const int* icpmat;
  double *cprho, *cpe, *cpp, *cpcs2, *cpvol, *frvol, *cpm, *frm, *cpvisc;
  d4 *cpviscx, *cpviscy, *cpfx, *cpfy;
  // ALE scratch
  d4 *fcdv, *fcdm, *eflux, *cndm, *cnflux, *cnfu, *cnfv, *cnm0, *cnmass_new;
  double *vpr, *mpr, *cutm_el;
  double* rscr25;            // split-advection stale-scratch emulation (unused)
  // dt reduction partials
  double* red_v;             // [2*nblk]
  int* red_i;                // [2*nblk]
  DevStep* step;
  StepRec* hist;
  // batch (null in a single-mesh context)
  DevStep* steps;            // [ninst] step headers
  const DevInst* inst;       // [ninst]
  const int* elinst;         // [nel] mesh of an element
  const int* ndinst;         // [nnd] mesh of a node
  const int* blkinst;        // [nblk_batch] mesh of a k_getdt block
  int ninst, nblk_batch;
  int nd_block;              // block size of the batch's node kernels (autotuned)
  // learned mixed-cell closure (bl_set_closure): 0 off, 1 volume and energy
  // exchange, 2 volume only
  int closure;
  float* mlp_img;            // the network's parameters as their shared-memory
                             // image (bl_mma.cuh), copied at bl_set_closure
  const float* mlp_norm;     // [22]: feature means, inverse spreads, output
                             // scale, conservation tolerance
  double* mxv0;              // [nmx] cell volume at the start of the step
  unsigned long long* mlp_count;  // [2]: cells the closure saw, cells it rejected
};

// ---------------------------------------------------------------- helpers

// Fortran MAX/MIN as the CPU restatement evaluates them, (b > a) ? b : a
// and (b < a) ? b : a: the first argument is returned on ties and when
// either is NaN.  The comparison runs on the integer pipe (bl_fp64.cuh).
__device__ __forceinline__ double maxF(double a, double b) { return gtF(b, a) ? b : a; }
__device__ __forceinline__ double minF(double a, double b) { return gtF(a, b) ? b : a; }
// the same, cheaper, when the sign bit is known to be clear (a square root,
// an absolute value, a sum of squares): of a for maxF_nn, of b for minF_nn
__device__ __forceinline__ double maxF_nn(double a, double b) { return gt_nn(b, a) ? b : a; }
__device__ __forceinline__ double minF_nn(double a, double b) { return gt_nn(a, b) ? b : a; }
// Fortran SIGN(a,b): |a| with the sign bit of b (negative zero honoured);
// signF itself is in bl_fp64.cuh, a sign-bit operation.

__device__ __forceinline__ int fc_of(int packed, int j) { return (packed >> (8 * j)) & 0xff; }

__device__ __forceinline__ double c4(const d4& v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

}  // namespace bl
