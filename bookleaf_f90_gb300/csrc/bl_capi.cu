// bl_capi.cu -- the C-ABI of include/bookleaf_gb300.h.
//
// Host side of the drop-in boundary: it owns the device mirrors of the
// dataAPI fields the hot path touches, the node->corner CSR tables, the
// device time-step state, and it sequences the kernels of bl_kernels.cu the
// way inf_solver_getdt / inf_solver_lagstep / inf_solver_alestep sequence
// the reference's loops.  No CPU fallback exists: every entry point fails
// when CUDA is not usable.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/bookleaf_gb300.h"
#include "bl_device.cuh"
#include "bl_ctx.h"
#include "bl_kernels.h"
#include "bl_mma.cuh"
#include "bl_setup.cuh"

using bl::DevStep;
using bl::d4;


namespace {

const bl::Launchers kFast = {bl::fast::getdt_blocks,          bl::fast::getdt_grid,
                             bl::fast::launch_getdt,
                             bl::fast::launch_lag_force,       bl::fast::launch_lag_accel,
                             bl::fast::launch_lag_state,       bl::fast::launch_ale,
                             bl::fast::launch_getdt_batch,     bl::fast::launch_lag_force_batch,
                             bl::fast::launch_lag_accel_batch, bl::fast::launch_lag_state_batch,
                             bl::fast::launch_ale_batch,       bl::fast::prepare_mix_closure,
                             bl::fast::launch_mix_closure,     bl::fast::launch_mix_closure_batch,
                             bl::fast::getdt_launches};
const bl::Launchers kExact = {bl::exact::getdt_blocks,          bl::exact::getdt_grid,
                              bl::exact::launch_getdt,
                              bl::exact::launch_lag_force,       bl::exact::launch_lag_accel,
                              bl::exact::launch_lag_state,       bl::exact::launch_ale,
                              bl::exact::launch_getdt_batch,     bl::exact::launch_lag_force_batch,
                              bl::exact::launch_lag_accel_batch, bl::exact::launch_lag_state_batch,
                              bl::exact::launch_ale_batch,       bl::exact::prepare_mix_closure,
                              bl::exact::launch_mix_closure,     bl::exact::launch_mix_closure_batch,
                              bl::exact::getdt_launches};
const bl::Launchers kMixed = {bl::mixed::getdt_blocks,          bl::mixed::getdt_grid,
                              bl::mixed::launch_getdt,
                              bl::mixed::launch_lag_force,       bl::mixed::launch_lag_accel,
                              bl::mixed::launch_lag_state,       bl::mixed::launch_ale,
                              bl::mixed::launch_getdt_batch,     bl::mixed::launch_lag_force_batch,
                              bl::mixed::launch_lag_accel_batch, bl::mixed::launch_lag_state_batch,
                              bl::mixed::launch_ale_batch,       bl::mixed::prepare_mix_closure,
                              bl::mixed::launch_mix_closure,     bl::mixed::launch_mix_closure_batch,
                              bl::mixed::getdt_launches};

// batches (defined with bl_init_batch below)
void batch_copy(bl_ctx* x, int id, bool to_mesh);


void set_err(bl_error* e, int ierr, int iout, const char* msg) {
  if (!e) return;
  e->ierr = ierr;
  e->iout = iout;
  std::strncpy(e->serr, msg ? msg : "", BL_SLEN);
  e->serr[BL_SLEN] = 0;
}

int cuda_fail(bl_error* e, cudaError_t r, const char* where) {
  char msg[BL_SLEN + 1];
  std::snprintf(msg, sizeof msg, "ERROR: CUDA %s in %s", cudaGetErrorString(r), where);
  set_err(e, BL_FAILURE, BL_HALT_ALL, msg);
  return BL_FAILURE;
}

// The single-mesh solver entry points and diagnostics refuse a batch
// context (its meshes each have their own time step: bl_run_batch).
bool reject_batch(bl_ctx* x, bl_error* e, const char* where) {
  if (!x || x->ninst == 0) return false;
  char msg[BL_SLEN + 1];
  std::snprintf(msg, sizeof msg, "ERROR: %s on a batch context (use bl_run_batch)", where);
  set_err(e, BL_FAILURE, BL_HALT_ALL, msg);
  return true;
}

// Device arrays come from a per-context arena: chunks of at least 64 MB
// (doubling), each allocated and zeroed once, carved in 256-byte aligned
// pieces, so that a context's few dozen arrays cost a handful of
// cudaMalloc calls instead of one each.  Every piece starts zeroed.
template <class T>
T* dalloc(bl_ctx* x, size_t n, cudaError_t& st) {
  if (n == 0) n = 1;
  const size_t bytes = (n * sizeof(T) + 255) & ~(size_t)255;
  if (x->arena_left < bytes) {
    size_t sz = x->arena_next < ((size_t)64 << 20) ? ((size_t)64 << 20) : x->arena_next;
    if (sz < bytes) sz = bytes;
    void* p = nullptr;
    cudaError_t r = cudaMalloc(&p, sz);
    if (r != cudaSuccess) {
      st = r;
      return nullptr;
    }
    cudaMemsetAsync(p, 0, sz, x->stream);
    x->bufs.push_back(p);
    x->arena_ptr = static_cast<char*>(p);
    x->arena_left = sz;
    x->arena_next = 2 * sz;
  }
  void* p = x->arena_ptr;
  x->arena_ptr += bytes;
  x->arena_left -= bytes;
  return static_cast<T*>(p);
}

template <class T>
void up(bl_ctx* x, T* d, const void* h, size_t n) {
  if (h && n) cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, x->stream);
}

// Fields copied back by bl_sync_to_host(ctx, 0): the state a host reader of
// the reference sees between solver calls.
const int kStateIds[] = {BL_ELDENSITY, BL_ELENERGY, BL_ELPRESSURE, BL_ELCS2, BL_ELVOLUME,
                         BL_A1, BL_A2, BL_A3, BL_B1, BL_B2, BL_B3, BL_CNWT, BL_CNX, BL_CNY,
                         BL_CNVISCX, BL_CNVISCY, BL_ELVISC, BL_ELMASS, BL_CNMASS, BL_NDX,
                         BL_NDY, BL_NDU, BL_NDV, BL_CPDENSITY, BL_CPENERGY, BL_CPPRESSURE,
                         BL_CPCS2, BL_CPVOLUME, BL_FRVOLUME, BL_CPA1, BL_CPA3, BL_CPB1,
                         BL_CPB3};

bool ale_active(const bl_config& c, double time) {  // ale_dr_utils.f90:35-51
  if (!c.ale_zexist) return false;
  return (time >= c.ale_mintime) && (time <= c.ale_maxtime);
}

const char* kSdt[5] = {" MAXIMUM", "  GROWTH", " INITIAL", "     CFL", "     DIV"};

void fill_ts_from_step(bl_ctx* x, const DevStep& S, bl_timestep* ts) {
  ts->nstep = S.nstep;
  ts->dt = S.dt;
  ts->time = S.time;
  ts->idtel = S.idtel;
  std::memset(ts->sdt, 0, sizeof ts->sdt);
  std::memcpy(ts->sdt, kSdt[S.sdt < 0 || S.sdt > 4 ? 0 : S.sdt], 8);
  std::memset(ts->mdt, 0, sizeof ts->mdt);
  // time_dr_setmaterial (time_dr_advance.f90:134-155)
  if (S.idtel > 0 && S.idtel <= x->s.nel) {
    int ii = x->ielmat_h[S.idtel - 1];
    if (ii > 0) {
      ts->imdt = ii;
      std::snprintf(ts->mdt, sizeof ts->mdt, "%10d", ii);
    } else {
      ts->imdt = 0;
      std::memcpy(ts->mdt, "     MIXED", 10);
    }
  } else {
    ts->imdt = -1;
    std::memcpy(ts->mdt, "   UNKNOWN", 10);
  }
}

bool same_bits(double a, double b) { return std::memcmp(&a, &b, sizeof a) == 0; }

// The step header the next kernels start from.  When the device already
// holds it -- the fields the kernels read (time, dt, 1/dt, nstep, idtel,
// the mode) are the same bits and every flag and accumulator the kernels
// set is clear -- the upload is skipped: a host that passes back the
// timestep the previous call returned saves one copy per call.
void header_from_ts(bl_ctx* x, const bl_timestep* ts, int run_mode) {
  DevStep h;
  std::memset(&h, 0, sizeof h);
  h.time = ts->time;
  h.dt = ts->dt;
  h.dts = ts->dts;
  h.rdt = 1.0 / ts->dt;  // IEEE division: the device's DIV(1.0, dt) bit for bit
  h.nstep = ts->nstep;
  h.idtel = ts->idtel;
  h.run_mode = run_mode;
  const DevStep& d = *x->hstep;
  const bool current = x->hstep_current && run_mode == 0 && d.run_mode == 0 &&
                       same_bits(d.time, h.time) && same_bits(d.dt, h.dt) &&
                       same_bits(d.rdt, h.rdt) && d.nstep == h.nstep && d.idtel == h.idtel &&
                       d.ierr == 0 && d.iout == 0 && d.err_code == 0 && d.negvol_pred == 0 &&
                       d.negvol_corr == 0 && d.negvol_ale == 0 && d.stop_next == 0 &&
                       d.halted == 0 && d.nrecord == 0 && d.ticket == 0;
  x->hstep_current = false;
  if (current) return;
  *x->hstep = h;
  cudaMemcpyAsync(x->F.step, x->hstep, sizeof(DevStep), cudaMemcpyHostToDevice, x->stream);
}

int fetch_header(bl_ctx* x, bl_error* e, const char* where) {
  cudaMemcpyAsync(x->hstep, x->F.step, sizeof(DevStep), cudaMemcpyDeviceToHost, x->stream);
  cudaError_t r = cudaStreamSynchronize(x->stream);
  if (r != cudaSuccess) return cuda_fail(e, r, where);
  r = cudaGetLastError();
  if (r != cudaSuccess) return cuda_fail(e, r, where);
  x->hstep_current = true;
  return BL_SUCCESS;
}

// The per-call entry points queue their kernels and the download of the
// step header as one replay of a graph captured on first use (again when
// the kernels' arguments change), then wait for it: one launch instead of
// one per kernel plus a copy, and the graph's back-to-back kernel launches.
enum { kCallGetdt = 0, kCallLagstep = 1, kCallAlestep = 2 };

void queue_call_kernels(bl_ctx* x, int which) {
  if (which == kCallGetdt) {
    x->L.getdt(x->F, x->C, x->stream);
  } else if (which == kCallLagstep) {
    x->L.lag_force(x->F, x->C, x->stream);
    x->L.lag_accel(x->F, x->C, x->stream);
    x->L.lag_state(x->F, x->C, x->stream);
    x->L.mix_closure(x->F, x->C, x->stream);
  } else {
    x->L.ale(x->F, x->C, x->stream);
  }
}

int run_call(bl_ctx* x, int which, bl_error* e, const char* where) {
  cudaError_t r;
  if (!x->call_exec[which] || std::memcmp(&x->call_F[which], &x->F, sizeof x->F) != 0 ||
      std::memcmp(&x->call_C[which], &x->C, sizeof x->C) != 0) {
    if (x->call_exec[which]) cudaGraphExecDestroy(x->call_exec[which]);
    x->call_exec[which] = nullptr;
    cudaGraph_t g;
    r = cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal);
    if (r != cudaSuccess) return cuda_fail(e, r, where);
    queue_call_kernels(x, which);
    cudaMemcpyAsync(x->hstep, x->F.step, sizeof(DevStep), cudaMemcpyDeviceToHost, x->stream);
    r = cudaStreamEndCapture(x->stream, &g);
    if (r != cudaSuccess) return cuda_fail(e, r, where);
    r = cudaGraphInstantiate(&x->call_exec[which], g, 0);
    cudaGraphDestroy(g);
    if (r != cudaSuccess) {
      x->call_exec[which] = nullptr;
      return cuda_fail(e, r, where);
    }
    x->call_F[which] = x->F;
    x->call_C[which] = x->C;
  }
  r = cudaGraphLaunch(x->call_exec[which], x->stream);
  if (r != cudaSuccess) return cuda_fail(e, r, where);
  r = cudaStreamSynchronize(x->stream);
  if (r != cudaSuccess) return cuda_fail(e, r, where);
  r = cudaGetLastError();
  if (r != cudaSuccess) return cuda_fail(e, r, where);
  x->hstep_current = true;
  return BL_SUCCESS;
}

int negvol_error(int code, bl_error* e) {
  set_err(e, -code, BL_HALT_SINGLE, "ERROR: negative volume in geometry_dr_getgeometry");
  return -code;
}

}  // namespace

extern "C" {

const char* bl_version(void) { return "bookleaf_gb300 1.0 (sm_103a)"; }

}  // extern "C"

namespace {

// Region and material tables of a batch, concatenated over its meshes (a
// batch may hold more of either than one control file's bound).
struct Tables {
  std::vector<double> kap, pm;
  std::vector<int> zd, zm;
  std::vector<int> et;        // [nmat+1]
  std::vector<double> ep;     // [(nmat+1)*6]
};

int init_impl(bl_ctx** out, const bl_sizes* sizes, const bl_config* config, void* const* dh,
              int fp_mode, bl_error* error, const Tables* T) {
  set_err(error, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (!out || !sizes || !config || !dh) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_init: null argument");
    return BL_FAILURE;
  }
  *out = nullptr;
  if (fp_mode != BL_FP_FAST && fp_mode != BL_FP_EXACT && fp_mode != BL_FP_MIXED) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_init: unknown fp_mode");
    return BL_FAILURE;
  }
  int ndev = 0;
  cudaError_t r = cudaGetDeviceCount(&ndev);
  if (r != cudaSuccess || ndev < 1) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: no CUDA device available for the hot path");
    return BL_FAILURE;
  }
  const bl_sizes& s = *sizes;
  const bl_config& c = *config;
  if (s.nel < 1 || s.nnd < 4 || s.nreg < 1 || (!T && s.nreg > BL_MAXREG) || s.nmat < 1 ||
      (!T && s.nmat > BL_MAXMAT) || s.ncp < 0 || s.nmx < 0) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_init: sizes out of range");
    return BL_FAILURE;
  }
  if (c.ale_zexist && !c.ale_zeul) {
    set_err(error, BL_FAILURE, BL_HALT_ALL,
            "ERROR: ALE requires zeul (the reference implements no other mesh motion)");
    return BL_FAILURE;
  }
  static const int needed[] = {BL_ELDENSITY, BL_ELENERGY, BL_ELPRESSURE, BL_ELCS2,
                               BL_ELVOLUME, BL_A1, BL_A3, BL_B1, BL_B3, BL_CNWT, BL_ELMASS,
                               BL_CNMASS, BL_NDX, BL_NDY, BL_NDU, BL_NDV, BL_INDTYPE,
                               BL_IELSORT1, BL_IELND, BL_IELEL, BL_IELFC, BL_IELMAT, BL_IELREG};
  for (int id : needed)
    if (!dh[id]) {
      char msg[BL_SLEN + 1];
      std::snprintf(msg, sizeof msg, "ERROR: bl_init: field %d not registered", id);
      set_err(error, BL_FAILURE, BL_HALT_ALL, msg);
      return BL_FAILURE;
    }
  if (c.zsp && !dh[BL_SPMASS]) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_init: spmass needed (zsp)");
    return BL_FAILURE;
  }
  const int nel = s.nel, nnd = s.nnd, ncp = s.ncp, nmx = s.nmx;
  const int* ielnd = static_cast<const int*>(dh[BL_IELND]);
  const int* ielel = static_cast<const int*>(dh[BL_IELEL]);
  const int* ielfc = static_cast<const int*>(dh[BL_IELFC]);
  const int* ielreg = static_cast<const int*>(dh[BL_IELREG]);
  const int* srt1 = static_cast<const int*>(dh[BL_IELSORT1]);
  const int* ielmat = static_cast<const int*>(dh[BL_IELMAT]);
  // Checks on the host, reported after the connectivity's (checked on the
  // device below): ielsort2 and the mixed-cell lists.
  const char* herr = nullptr;
  if (c.ale_zexist) {
    const int* srt2 = static_cast<const int*>(dh[BL_IELSORT2]);
    if (!srt2) {
      herr = "ERROR: bl_init: ielsort2 needed for ALE";
    } else {
      // serial BookLeaf sets ielsort2 to the identity (init_dr_utils.f90:65-68);
      // ale_kn_updatend sums in natural order, calcbasisnd in ielsort2 order
      for (int i = 0; i < nel && !herr; i++)
        if (srt2[i] != i + 1) herr = "ERROR: bl_init: ielsort2 must be the identity for one partition";
    }
  }
  std::vector<int> elmx(nel, -1);
  if (ncp > 0 && !herr) {
    const int* imxel = static_cast<const int*>(dh[BL_IMXEL]);
    const int* imxfcp = static_cast<const int*>(dh[BL_IMXFCP]);
    const int* imxncp = static_cast<const int*>(dh[BL_IMXNCP]);
    const int* icpmat = static_cast<const int*>(dh[BL_ICPMAT]);
    static const int cpneed[] = {BL_CPDENSITY, BL_CPENERGY, BL_CPPRESSURE, BL_CPCS2, BL_CPVOLUME,
                                 BL_FRVOLUME, BL_CPMASS, BL_FRMASS};
    bool ok = imxel && imxfcp && imxncp && icpmat;
    for (int id : cpneed) ok = ok && dh[id];
    if (!ok) herr = "ERROR: bl_init: component fields missing";
    for (int m = 0; m < nmx && !herr; m++) {
      if (imxel[m] < 1 || imxel[m] > nel || imxfcp[m] < 1 || imxncp[m] < 1 ||
          imxfcp[m] + imxncp[m] - 1 > ncp)
        herr = "ERROR: bl_init: mixed-cell lists out of range";
      else
        elmx[imxel[m] - 1] = m;
    }
    for (int k = 0; k < ncp && !herr; k++)
      if (icpmat[k] < 0 || icpmat[k] > s.nmat) herr = "ERROR: bl_init: icpmat out of range";
  }

  bl_ctx* x = new bl_ctx();
  x->s = s;
  x->c = c;
  x->fp_mode = fp_mode;
  x->L = (fp_mode == BL_FP_EXACT) ? kExact : (fp_mode == BL_FP_MIXED) ? kMixed : kFast;
  for (int id = 1; id <= BL_NID; id++) x->host[id] = dh[id];
  x->ielmat_h.assign(ielmat, ielmat + nel);
  cudaGetDevice(&x->device);
  r = cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking);
  if (r != cudaSuccess) {
    delete x;
    return cuda_fail(error, r, "bl_init");
  }
  cudaError_t st = cudaSuccess;
  bl::DevFields& F = x->F;
  F.nel = nel;
  F.nnd = nnd;
  F.ncp = ncp;
  F.nmx = nmx;
  // ---- connectivity: uploaded as the caller holds it, checked and
  // converted to 0-based on the device (bl_setup.cuh); nothing indexes
  // with it before the host has read the check's error bits
  {
    namespace su = bl::setup;
    int4* d_nd = dalloc<int4>(x, nel, st);
    int4* d_ee = dalloc<int4>(x, nel, st);
    int* d_fc = dalloc<int>(x, nel, st);
    int* d_rg = dalloc<int>(x, nel, st);
    int* d_mt = dalloc<int>(x, nel, st);
    int* d_it = dalloc<int>(x, nnd, st);
    int* d_off = dalloc<int>(x, nnd + 1, st);
    int* d_ent = dalloc<int>(x, 4L * nel, st);
    // set-up scratch (stays with the context's arena: 8 bytes an element
    // and 4 a node): ielsort1, its permutation counts, the node cursors,
    // the scan's tile sums, the error bits
    const int nb = su::blocks_for(nnd, su::kScanTile);
    int* d_srt = dalloc<int>(x, nel, st);
    int* d_seen = dalloc<int>(x, nel, st);
    int* d_cnt = dalloc<int>(x, nnd, st);
    int* d_bsum = dalloc<int>(x, nb, st);
    int* d_bad = dalloc<int>(x, 1, st);
    if (st != cudaSuccess) goto fail;
    up(x, d_nd, ielnd, nel);  // four nodes an element, as one int4
    up(x, d_ee, ielel, nel);
    up(x, reinterpret_cast<int4*>(d_ent), ielfc, nel);  // the faces, until the fill
    up(x, d_rg, ielreg, nel);
    up(x, d_mt, ielmat, nel);
    up(x, d_it, dh[BL_INDTYPE], nnd);
    up(x, d_srt, srt1, nel);
    const int ge = su::blocks_for(nel, su::kThreads), gn = su::blocks_for(nnd, su::kThreads);
    su::k_check_pack<<<ge, su::kThreads, 0, x->stream>>>(
        d_nd, d_ee, reinterpret_cast<const int4*>(d_ent), d_fc, d_rg, d_srt, d_mt, d_seen, nel,
        nnd, s.nreg, s.nmat, d_bad);
    int bad = 0;
    cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, x->stream);
    r = cudaStreamSynchronize(x->stream);
    if (r == cudaSuccess) r = cudaGetLastError();
    if (r != cudaSuccess) {
      st = r;
      goto fail;
    }
    if (bad || herr) {
      bl_finalize(x);
      set_err(error, BL_FAILURE, BL_HALT_ALL,
              (bad & su::kBadConn)      ? "ERROR: bl_init: connectivity out of range"
              : (bad & su::kBadRegSort) ? "ERROR: bl_init: ielreg/ielsort1 out of range"
              : (bad & su::kBadPerm)    ? "ERROR: bl_init: ielsort1 is not a permutation"
              : (bad & su::kBadMat)     ? "ERROR: bl_init: ielmat out of range"
                                        : herr);
      return BL_FAILURE;
    }
    F.ielnd = d_nd;
    F.ielel = d_ee;
    F.ielfc = d_fc;
    F.ielreg = d_rg;
    F.ielmat = d_mt;
    F.indtype = d_it;
    // node -> corner tables: counts and offsets (shared by both tables)
    su::k_count<<<ge, su::kThreads, 0, x->stream>>>(d_nd, nel, nnd, d_cnt);
    su::k_scan_tiles<<<nb, su::kThreads, 0, x->stream>>>(d_cnt, nnd, d_bsum);
    su::k_scan_sums<<<1, su::kThreads, 0, x->stream>>>(d_bsum, nb);
    su::k_scan_apply<<<nb, su::kThreads, 0, x->stream>>>(d_cnt, nnd, d_bsum, d_off);
    // corner-major, hydro_kn_scatteracceleration's order: corner jj outer,
    // elements in ielsort1 order inner (hydro_kn_getacceleration.f90:53-72)
    su::k_fill<<<ge, su::kThreads, 0, x->stream>>>(d_nd, d_srt, nel, nnd, d_cnt, d_ent);
    su::k_sort<<<gn, su::kThreads, 0, x->stream>>>(d_off, d_srt, nel, nnd, d_ent);
    F.nc_off = d_off;
    F.nc_ent = d_ent;
    // element-major, natural order (ale_kn_calcbasisnd / massbasisnd / updatend)
    if (c.ale_zexist) {
      int* d_ent2 = dalloc<int>(x, 4L * nel, st);
      if (st != cudaSuccess) goto fail;
      su::k_copy<<<gn, su::kThreads, 0, x->stream>>>(d_off, nnd, d_cnt);
      su::k_fill<<<ge, su::kThreads, 0, x->stream>>>(d_nd, nullptr, nel, nnd, d_cnt, d_ent2);
      su::k_sort<<<gn, su::kThreads, 0, x->stream>>>(d_off, nullptr, nel, nnd, d_ent2);
      F.ne_off = d_off;
      F.ne_ent = d_ent2;
    }
    r = cudaGetLastError();
    if (r != cudaSuccess) {
      st = r;
      goto fail;
    }
  }
  // ---- node fields
  F.ndx = dalloc<double>(x, nnd, st);
  F.ndy = dalloc<double>(x, nnd, st);
  F.ndu = dalloc<double>(x, nnd, st);
  F.ndv = dalloc<double>(x, nnd, st);
  F.ndubar = dalloc<double>(x, nnd, st);
  F.ndvbar = dalloc<double>(x, nnd, st);
  // ---- element fields
  F.rho = dalloc<double>(x, nel, st);
  F.e = dalloc<double>(x, nel, st);
  F.p = dalloc<double>(x, nel, st);
  F.cs2 = dalloc<double>(x, nel, st);
  F.cs2v = dalloc<double>(x, nel, st);
  F.vol = dalloc<double>(x, nel, st);
  F.mass = dalloc<double>(x, nel, st);
  F.visc = dalloc<double>(x, nel, st);
  F.a1 = dalloc<double>(x, nel, st);
  F.a2 = dalloc<double>(x, nel, st);
  F.a3 = dalloc<double>(x, nel, st);
  F.b1 = dalloc<double>(x, nel, st);
  F.b2 = dalloc<double>(x, nel, st);
  F.b3 = dalloc<double>(x, nel, st);
  F.rho_h = dalloc<double>(x, nel, st);
  F.cnwt = dalloc<d4>(x, nel, st);
  F.cnmass = dalloc<d4>(x, nel, st);
  F.cnviscx = dalloc<d4>(x, nel, st);
  F.cnviscy = dalloc<d4>(x, nel, st);
  F.cnfx = dalloc<d4>(x, nel, st);
  F.cnfy = dalloc<d4>(x, nel, st);
  F.cnwt_h = dalloc<d4>(x, nel, st);
  if (c.zsp) F.spmass = dalloc<d4>(x, nel, st);
  if (c.ale_zexist) {
    F.fcdv = dalloc<d4>(x, nel, st);
    F.fcdm = dalloc<d4>(x, nel, st);
    F.eflux = dalloc<d4>(x, nel, st);
    F.cnflux = dalloc<d4>(x, nel, st);
    F.cnfu = dalloc<d4>(x, nel, st);
    F.cnfv = dalloc<d4>(x, nel, st);
    F.vpr = dalloc<double>(x, nel, st);
    F.mpr = dalloc<double>(x, nel, st);
    F.cutm_el = dalloc<double>(x, nel, st);
  }
  {
    const int nblk = x->L.getdt_grid(nel);
    F.red_v = dalloc<double>(x, 2L * nblk, st);
    F.red_i = dalloc<int>(x, 2L * nblk, st);
  }
  F.step = dalloc<DevStep>(x, 1, st);
  if (st != cudaSuccess) goto fail;
  if (cudaMallocHost(&x->hstep, sizeof(DevStep)) != cudaSuccess) {
    st = cudaErrorMemoryAllocation;
    goto fail;
  }
  std::memset(x->hstep, 0, sizeof(DevStep));
  up(x, F.ndx, dh[BL_NDX], nnd);
  up(x, F.ndy, dh[BL_NDY], nnd);
  up(x, F.ndu, dh[BL_NDU], nnd);
  up(x, F.ndv, dh[BL_NDV], nnd);
  up(x, F.rho, dh[BL_ELDENSITY], nel);
  up(x, F.e, dh[BL_ELENERGY], nel);
  up(x, F.p, dh[BL_ELPRESSURE], nel);
  up(x, F.cs2, dh[BL_ELCS2], nel);
  up(x, F.vol, dh[BL_ELVOLUME], nel);
  up(x, F.mass, dh[BL_ELMASS], nel);
  up(x, F.visc, dh[BL_ELVISC], nel);
  up(x, F.a1, dh[BL_A1], nel);
  up(x, F.a2, dh[BL_A2], nel);
  up(x, F.a3, dh[BL_A3], nel);
  up(x, F.b1, dh[BL_B1], nel);
  up(x, F.b2, dh[BL_B2], nel);
  up(x, F.b3, dh[BL_B3], nel);
  up(x, F.cnwt, dh[BL_CNWT], nel);
  up(x, F.cnmass, dh[BL_CNMASS], nel);
  up(x, F.cnviscx, dh[BL_CNVISCX], nel);
  up(x, F.cnviscy, dh[BL_CNVISCY], nel);
  if (c.zsp) up(x, F.spmass, dh[BL_SPMASS], nel);
  // ---- mixed cells
  if (ncp > 0) {
    std::vector<int> mxel(nmx), mxf(nmx);
    const int* imxel = static_cast<const int*>(dh[BL_IMXEL]);
    const int* imxfcp = static_cast<const int*>(dh[BL_IMXFCP]);
    for (int m = 0; m < nmx; m++) {
      mxel[m] = imxel[m] - 1;
      mxf[m] = imxfcp[m] - 1;
    }
    int* d_elmx = dalloc<int>(x, nel, st);
    int* d_mxel = dalloc<int>(x, nmx, st);
    int* d_mxf = dalloc<int>(x, nmx, st);
    int* d_mxn = dalloc<int>(x, nmx, st);
    int* d_cpm = dalloc<int>(x, ncp, st);
    F.cprho = dalloc<double>(x, ncp, st);
    F.cpe = dalloc<double>(x, ncp, st);
    F.cpp = dalloc<double>(x, ncp, st);
    F.cpcs2 = dalloc<double>(x, ncp, st);
    F.cpvol = dalloc<double>(x, ncp, st);
    F.frvol = dalloc<double>(x, ncp, st);
    F.cpm = dalloc<double>(x, ncp, st);
    F.frm = dalloc<double>(x, ncp, st);
    F.cpvisc = dalloc<double>(x, ncp, st);
    F.cpviscx = dalloc<d4>(x, ncp, st);
    F.cpviscy = dalloc<d4>(x, ncp, st);
    F.cpfx = dalloc<d4>(x, ncp, st);
    F.cpfy = dalloc<d4>(x, ncp, st);
    if (st != cudaSuccess) goto fail;
    up(x, d_elmx, elmx.data(), nel);
    up(x, d_mxel, mxel.data(), nmx);
    up(x, d_mxf, mxf.data(), nmx);
    up(x, d_mxn, dh[BL_IMXNCP], nmx);
    up(x, d_cpm, dh[BL_ICPMAT], ncp);
    up(x, F.cprho, dh[BL_CPDENSITY], ncp);
    up(x, F.cpe, dh[BL_CPENERGY], ncp);
    up(x, F.cpp, dh[BL_CPPRESSURE], ncp);
    up(x, F.cpcs2, dh[BL_CPCS2], ncp);
    up(x, F.cpvol, dh[BL_CPVOLUME], ncp);
    up(x, F.frvol, dh[BL_FRVOLUME], ncp);
    up(x, F.cpm, dh[BL_CPMASS], ncp);
    up(x, F.frm, dh[BL_FRMASS], ncp);
    // component viscosity is zeroed at start and never set (hydro_dr_init.f90:48-51;
    // hydro_kn_getcpeviscosity is empty), so its device copies stay zero
    F.elmx = d_elmx;
    F.imxel = d_mxel;
    F.imxfcp = d_mxf;
    F.imxncp = d_mxn;
    F.icpmat = d_cpm;
    cudaStreamSynchronize(x->stream);
  }
  // ---- configuration tables
  {
    bl::DevCfg& C = x->C;
    C.cvisc1 = c.cvisc1;
    C.cvisc2 = c.cvisc2;
    C.cfl_sf = c.cfl_sf;
    C.div_sf = c.div_sf;
    C.zcut = c.zcut;
    C.zerocut = c.zerocut;
    C.dencut = c.dencut;
    C.accut = c.accut;
    C.ccut = c.ccut;
    C.pcut = c.pcut;
    C.dt_g = c.dt_g;
    C.dt_min = c.dt_min;
    C.dt_max = c.dt_max;
    C.dt_initial = c.dt_initial;
    C.time_end = c.time_end;
    C.ale_mintime = c.ale_mintime;
    C.ale_maxtime = c.ale_maxtime;
    C.ztq = c.ztq;
    C.zhg = c.zhg;
    C.zsp = c.zsp;
    C.nreg = s.nreg;
    C.nmat = s.nmat;
    C.ale_zexist = c.ale_zexist;
    C.ale_zeul = c.ale_zeul;
    C.adv_type = c.ale_adv_type;
    const int nr = s.nreg, nm = s.nmat + 1;
    std::vector<double> kap, pm, ep;
    std::vector<int> zd, zm, et;
    if (T) {
      kap = T->kap;
      pm = T->pm;
      zd = T->zd;
      zm = T->zm;
      et = T->et;
      ep = T->ep;
    } else {
      kap.assign(c.kappareg, c.kappareg + nr);
      pm.assign(c.pmeritreg, c.pmeritreg + nr);
      zd.assign(c.zdtnotreg, c.zdtnotreg + nr);
      zm.assign(c.zmidlength, c.zmidlength + nr);
      et.assign(c.eos_type, c.eos_type + nm);
      ep.resize(6L * nm);
      for (int m = 0; m < nm; m++)
        for (int k = 0; k < 6; k++) ep[6 * m + k] = c.eos_param[m][k];
    }
    std::vector<double> gm1(nm), ggm1(nm);
    for (int m = 0; m < nm; m++) {
      gm1[m] = ep[6 * m] - 1.0;
      ggm1[m] = ep[6 * m] * (ep[6 * m] - 1.0);
    }
    double* d_kap = dalloc<double>(x, nr, st);
    double* d_pm = dalloc<double>(x, nr, st);
    int* d_zd = dalloc<int>(x, nr, st);
    int* d_zm = dalloc<int>(x, nr, st);
    int* d_et = dalloc<int>(x, nm, st);
    double* d_ep = dalloc<double>(x, 6L * nm, st);
    double* d_g1 = dalloc<double>(x, nm, st);
    double* d_g2 = dalloc<double>(x, nm, st);
    if (st != cudaSuccess) goto fail;
    up(x, d_kap, kap.data(), nr);
    up(x, d_pm, pm.data(), nr);
    up(x, d_zd, zd.data(), nr);
    up(x, d_zm, zm.data(), nr);
    up(x, d_et, et.data(), nm);
    up(x, d_ep, ep.data(), 6L * nm);
    up(x, d_g1, gm1.data(), nm);
    up(x, d_g2, ggm1.data(), nm);
    C.kappareg = d_kap;
    C.pmeritreg = d_pm;
    C.zdtnotreg = d_zd;
    C.zmidlength = d_zm;
    C.eos_type = d_et;
    C.eos_param = d_ep;
    C.eos_gm1 = d_g1;
    C.eos_ggm1 = d_g2;
    cudaStreamSynchronize(x->stream);
  }
  r = cudaStreamSynchronize(x->stream);
  if (r != cudaSuccess) {
    st = r;
    goto fail;
  }
  *out = x;
  return BL_SUCCESS;
fail:
  bl_finalize(x);
  return cuda_fail(error, st == cudaSuccess ? cudaErrorMemoryAllocation : st, "bl_init");
}

}  // namespace

extern "C" {

int bl_init(bl_ctx** out, const bl_sizes* sizes, const bl_config* config, void* const* dh,
            int fp_mode, bl_error* error) {
  return init_impl(out, sizes, config, dh, fp_mode, error, nullptr);
}

int bl_finalize(bl_ctx* x) {
  if (!x) return BL_SUCCESS;
  if (x->stream) cudaStreamSynchronize(x->stream);
  if (x->gexec) cudaGraphExecDestroy(x->gexec);
  if (x->bexec) cudaGraphExecDestroy(x->bexec);
  for (auto& g : x->call_exec)
    if (g) cudaGraphExecDestroy(g);
  if (x->hsteps) cudaFreeHost(x->hsteps);
  for (void* p : x->bufs) cudaFree(p);
  if (x->F.hist) cudaFree(x->F.hist);
  if (x->diag) cudaFree(x->diag);
  if (x->hstep) cudaFreeHost(x->hstep);
  if (x->stream) cudaStreamDestroy(x->stream);
  delete x;
  return BL_SUCCESS;
}

int bl_getdt(bl_ctx* x, bl_timestep* ts, bl_error* e) {
  set_err(e, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (reject_batch(x, e, "bl_getdt")) return BL_FAILURE;
  if (!x || !ts) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_getdt: null argument");
    return BL_FAILURE;
  }
  header_from_ts(x, ts, 0);
  x->launches += x->L.getdt_launches(x->C);
  int rc = run_call(x, kCallGetdt, e, "bl_getdt");
  if (rc != BL_SUCCESS) return rc;
  x->cs2_is_v = true;
  const DevStep& S = *x->hstep;
  if (S.err_code == 1) {
    set_err(e, BL_FAILURE, BL_HALT_SINGLE, "ERROR: negative CFL condition in hydro_dr_getdt");
    return BL_FAILURE;
  }
  fill_ts_from_step(x, S, ts);
  if (S.err_code == 2) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: dt < dt_min");
    return BL_FAILURE;
  }
  return BL_SUCCESS;
}

int bl_lagstep(bl_ctx* x, bl_timestep* ts, bl_error* e) {
  set_err(e, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (reject_batch(x, e, "bl_lagstep")) return BL_FAILURE;
  if (!x || !ts) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_lagstep: null argument");
    return BL_FAILURE;
  }
  header_from_ts(x, ts, 0);
  x->launches += bl::launches_lagstep(x->F);
  int rc = run_call(x, kCallLagstep, e, "bl_lagstep");
  if (rc != BL_SUCCESS) return rc;
  x->cs2_is_v = false;
  // time_dr_setpredictor / setcorrector leave the corrector state behind
  ts->zcorrector = 1;
  ts->dts = ts->dt;
  const DevStep& S = *x->hstep;
  if (S.negvol_pred) return negvol_error(S.negvol_pred, e);
  if (S.negvol_corr) return negvol_error(S.negvol_corr, e);
  return BL_SUCCESS;
}

int bl_alestep(bl_ctx* x, const bl_timestep* ts, bl_error* e) {
  set_err(e, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (reject_batch(x, e, "bl_alestep")) return BL_FAILURE;
  if (!x || !ts) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_alestep: null argument");
    return BL_FAILURE;
  }
  if (!ale_active(x->c, ts->time)) return BL_SUCCESS;
  if (x->c.ale_adv_type != 1) {
    set_err(e, BL_FAILURE, BL_HALT_ALL,
            x->c.ale_adv_type == 2 ? "ERROR: adv_type 2 (split) not supported on the device"
                                   : "ERROR: unrecognised adv_type");
    return BL_FAILURE;
  }
  header_from_ts(x, ts, 0);
  x->launches += bl::kLaunchesAle;
  int rc = run_call(x, kCallAlestep, e, "bl_alestep");
  if (rc != BL_SUCCESS) return rc;
  const DevStep& S = *x->hstep;
  if (S.negvol_ale) return negvol_error(S.negvol_ale, e);
  return BL_SUCCESS;
}

int bl_run(bl_ctx* x, bl_timestep* ts, int max_steps, bl_step_record* history, int* nsteps,
           bl_error* e) {
  set_err(e, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (reject_batch(x, e, "bl_run")) return BL_FAILURE;
  if (nsteps) *nsteps = 0;
  if (!x || !ts || max_steps < 0) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_run: bad argument");
    return BL_FAILURE;
  }
  if (max_steps == 0) return BL_SUCCESS;
  if (x->c.ale_zexist && x->c.ale_adv_type != 1) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_run: only adv_type 1 runs on the device");
    return BL_FAILURE;
  }
  cudaError_t r;
  if (history && max_steps > x->hist_cap) {
    if (x->F.hist) cudaFree(x->F.hist);
    x->F.hist = nullptr;
    r = cudaMalloc(&x->F.hist, sizeof(bl::StepRec) * (size_t)max_steps);
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run");
    x->hist_cap = max_steps;
  }
  // the kernels of this run see the history buffer only when one is wanted
  bl::DevFields F = x->F;
  bl::DevCfg C = x->C;
  if (!history) F.hist = nullptr;
  C.max_records = history ? x->hist_cap : 0;
  const bool with_ale = x->c.ale_zexist != 0;
  const int G = 16;  // steps per graph launch
  if (!x->gexec || x->gsteps != G || x->g_ale != with_ale || x->g_hist != F.hist ||
      x->g_maxrec != C.max_records) {
    if (x->gexec) cudaGraphExecDestroy(x->gexec);
    x->gexec = nullptr;
    cudaGraph_t g;
    r = cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal);
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run capture");
    for (int k = 0; k < G; k++) {
      x->L.getdt(F, C, x->stream);
      x->L.lag_force(F, C, x->stream);
      x->L.lag_accel(F, C, x->stream);
      x->L.lag_state(F, C, x->stream);
      x->L.mix_closure(F, C, x->stream);
      if (with_ale) x->L.ale(F, C, x->stream);
    }
    r = cudaStreamEndCapture(x->stream, &g);
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run capture");
    r = cudaGraphInstantiate(&x->gexec, g, 0);
    cudaGraphDestroy(g);
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run instantiate");
    x->gsteps = G;
    x->g_ale = with_ale;
    x->g_hist = F.hist;
    x->g_maxrec = C.max_records;
  }
  header_from_ts(x, ts, 1);
  // step limit: getdt stops once nrecord reaches it (DevStep.nrecord counts)
  int launched = 0;
  const int per_step = x->L.getdt_launches(x->C) + bl::launches_lagstep(x->F) + (with_ale ? bl::kLaunchesAle : 0);
  int done = 0;
  while (true) {
    const int remaining = max_steps - done;
    if (remaining <= 0) break;
    if (remaining >= G) {
      r = cudaGraphLaunch(x->gexec, x->stream);
      if (r != cudaSuccess) return cuda_fail(e, r, "bl_run launch");
      x->launches += (long long)G * per_step;
      launched += G;
    } else {
      for (int k = 0; k < remaining; k++) {
        x->L.getdt(F, C, x->stream);
        x->L.lag_force(F, C, x->stream);
        x->L.lag_accel(F, C, x->stream);
        x->L.lag_state(F, C, x->stream);
        x->L.mix_closure(F, C, x->stream);
        if (with_ale) x->L.ale(F, C, x->stream);
      }
      x->launches += (long long)remaining * per_step;
      launched += remaining;
    }
    int rc = fetch_header(x, e, "bl_run");
    if (rc != BL_SUCCESS) return rc;
    done = x->hstep->nrecord;
    if (x->hstep->halted || x->hstep->stop_next || x->hstep->err_code ||
        x->hstep->negvol_pred || x->hstep->negvol_corr || x->hstep->negvol_ale)
      break;
    if (done >= max_steps) break;
  }
  const DevStep S = *x->hstep;
  const int nrec = std::min(S.nrecord, max_steps);
  if (nsteps) *nsteps = nrec;
  if (history && nrec > 0) {
    std::vector<bl::StepRec> tmp(nrec);
    r = cudaMemcpy(tmp.data(), F.hist, sizeof(bl::StepRec) * nrec, cudaMemcpyDeviceToHost);
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run history");
    for (int i = 0; i < nrec; i++) {
      history[i].time = tmp[i].time;
      history[i].dt = tmp[i].dt;
      history[i].nstep = tmp[i].nstep;
      history[i].idtel = tmp[i].idtel;
      history[i].sdt_code = tmp[i].sdt_code;
      history[i].ierr = tmp[i].ierr;
    }
  }
  x->cs2_is_v = false;
  fill_ts_from_step(x, S, ts);
  ts->zcorrector = 1;
  ts->dts = ts->dt;
  (void)launched;
  if (S.err_code == 1) {
    set_err(e, BL_FAILURE, BL_HALT_SINGLE, "ERROR: negative CFL condition in hydro_dr_getdt");
    return BL_FAILURE;
  }
  if (S.err_code == 2) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: dt < dt_min");
    return BL_FAILURE;
  }
  if (S.negvol_pred) return negvol_error(S.negvol_pred, e);
  if (S.negvol_corr) return negvol_error(S.negvol_corr, e);
  if (S.negvol_ale) return negvol_error(S.negvol_ale, e);
  return BL_SUCCESS;
}

// Per-kernel durations of the Lagrangian step: the four kernels of nstep
// steps are queued back to back with an event between each (the per-call
// path's header, so the end time does not stop them), then timed from the
// events once the last one has completed.
int bl_time_step_kernels(bl_ctx* x, bl_timestep* ts, int nstep, double* ms, int n, bl_error* e) {
  set_err(e, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (reject_batch(x, e, "bl_time_step_kernels")) return BL_FAILURE;
  constexpr int kMaxSteps = 64;
  if (!x || !ts || !ms || n < 4 || nstep < 1 || nstep > kMaxSteps) {
    set_err(e, BL_FAILURE, BL_HALT_ALL,
            "ERROR: bl_time_step_kernels: bad argument (nstep 1..64, n >= 4)");
    return BL_FAILURE;
  }
  std::vector<cudaEvent_t> ev(4 * nstep + 1, nullptr);
  cudaError_t r = cudaSuccess;
  for (auto& v : ev)
    if (r == cudaSuccess) r = cudaEventCreate(&v);
  auto release = [&]() {
    for (auto& v : ev)
      if (v) cudaEventDestroy(v);
  };
  if (r != cudaSuccess) {
    release();
    return cuda_fail(e, r, "bl_time_step_kernels");
  }
  header_from_ts(x, ts, 0);
  cudaEventRecord(ev[0], x->stream);
  for (int k = 0; k < nstep; k++) {
    x->L.getdt(x->F, x->C, x->stream);
    cudaEventRecord(ev[4 * k + 1], x->stream);
    x->L.lag_force(x->F, x->C, x->stream);
    cudaEventRecord(ev[4 * k + 2], x->stream);
    x->L.lag_accel(x->F, x->C, x->stream);
    cudaEventRecord(ev[4 * k + 3], x->stream);
    x->L.lag_state(x->F, x->C, x->stream);
    x->L.mix_closure(x->F, x->C, x->stream);
    cudaEventRecord(ev[4 * k + 4], x->stream);
  }
  x->launches += (long long)nstep * (x->L.getdt_launches(x->C) + bl::launches_lagstep(x->F));
  r = cudaEventSynchronize(ev[4 * nstep]);
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k = 0; k < nstep && r == cudaSuccess; k++)
    for (int j = 0; j < 4 && r == cudaSuccess; j++) {
      float t = 0.0f;
      r = cudaEventElapsedTime(&t, ev[4 * k + j], ev[4 * k + j + 1]);
      acc[j] += t;
    }
  release();
  if (r != cudaSuccess) return cuda_fail(e, r, "bl_time_step_kernels");
  for (int j = 0; j < 4; j++) ms[j] = acc[j] / nstep;
  int rc = fetch_header(x, e, "bl_time_step_kernels");
  if (rc != BL_SUCCESS) return rc;
  const DevStep S = *x->hstep;
  x->cs2_is_v = false;
  fill_ts_from_step(x, S, ts);
  ts->zcorrector = 1;
  ts->dts = ts->dt;
  if (S.err_code == 1) {
    set_err(e, BL_FAILURE, BL_HALT_SINGLE, "ERROR: negative CFL condition in hydro_dr_getdt");
    return BL_FAILURE;
  }
  if (S.err_code == 2) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: dt < dt_min");
    return BL_FAILURE;
  }
  if (S.negvol_pred) return negvol_error(S.negvol_pred, e);
  if (S.negvol_corr) return negvol_error(S.negvol_corr, e);
  return BL_SUCCESS;
}

// corner coordinates: out[e] = the element's four node values (the host's
// (4, nel) corner layout)
__global__ void k_cngather(const int4* __restrict__ ielnd, const double* __restrict__ nd,
                           int nel, d4* __restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  const int4 n = ielnd[e];
  out[e] = bl::make_d4(nd[n.x], nd[n.y], nd[n.z], nd[n.w]);
}

static size_t field_count(const bl_ctx* x, int id, int& kind) {
  // kind: 0 double element, 1 double corner, 2 double node, 3 double comp,
  //       4 derived (cnx/cny/cpa*), -1 not a device state field
  const int nel = x->s.nel, nnd = x->s.nnd, ncp = x->s.ncp;
  switch (id) {
    case BL_ELDENSITY: case BL_ELENERGY: case BL_ELPRESSURE: case BL_ELCS2: case BL_ELVOLUME:
    case BL_A1: case BL_A2: case BL_A3: case BL_B1: case BL_B2: case BL_B3: case BL_ELVISC:
    case BL_ELMASS:
      kind = 0;
      return nel;
    case BL_CNWT: case BL_CNVISCX: case BL_CNVISCY: case BL_CNMASS:
      kind = 1;
      return 4L * nel;
    case BL_NDX: case BL_NDY: case BL_NDU: case BL_NDV:
      kind = 2;
      return nnd;
    case BL_CPDENSITY: case BL_CPENERGY: case BL_CPPRESSURE: case BL_CPCS2: case BL_CPVOLUME:
    case BL_FRVOLUME:  // changes only under the learned closure
      kind = ncp > 0 ? 3 : -1;
      return ncp;
    case BL_CNX: case BL_CNY:
      kind = 4;
      return 4L * nel;
    case BL_CPA1: case BL_CPA3: case BL_CPB1: case BL_CPB3:
      kind = ncp > 0 ? 4 : -1;
      return ncp;
    default:
      kind = -1;
      return 0;
  }
}

static void* dev_ptr(bl_ctx* x, int id) {
  bl::DevFields& F = x->F;
  switch (id) {
    case BL_ELDENSITY: return F.rho;
    case BL_ELENERGY: return F.e;
    case BL_ELPRESSURE: return F.p;
    case BL_ELCS2: return x->cs2_is_v ? F.cs2v : F.cs2;
    case BL_ELVOLUME: return F.vol;
    case BL_A1: return F.a1;
    case BL_A2: return F.a2;
    case BL_A3: return F.a3;
    case BL_B1: return F.b1;
    case BL_B2: return F.b2;
    case BL_B3: return F.b3;
    case BL_ELVISC: return F.visc;
    case BL_ELMASS: return F.mass;
    case BL_CNWT: return F.cnwt;
    case BL_CNVISCX: return F.cnviscx;
    case BL_CNVISCY: return F.cnviscy;
    case BL_CNMASS: return F.cnmass;
    case BL_NDX: return F.ndx;
    case BL_NDY: return F.ndy;
    case BL_NDU: return F.ndu;
    case BL_NDV: return F.ndv;
    case BL_CPDENSITY: return F.cprho;
    case BL_CPENERGY: return F.cpe;
    case BL_CPPRESSURE: return F.cpp;
    case BL_CPCS2: return F.cpcs2;
    case BL_CPVOLUME: return F.cpvol;
    case BL_FRVOLUME: return F.frvol;
    default: return nullptr;
  }
}

int bl_sync_to_host(bl_ctx* x, int id) {
  if (!x) return BL_FAILURE;
  if (id != 0 && (id < 1 || id > BL_NID)) return BL_SUCCESS;
  const int* ids = id == 0 ? kStateIds : &id;
  const int nids = id == 0 ? (int)(sizeof kStateIds / sizeof kStateIds[0]) : 1;
  // every copy queued on the context's stream, one wait for all of them;
  // the corner coordinates (utils_kn_cngather of the node positions) are
  // gathered on the device first
  bool gathered_cp = false;
  for (int k = 0; k < nids; k++) {
    const int f = ids[k];
    if (!x->host[f]) continue;
    int kind;
    const size_t n = field_count(x, f, kind);
    if (kind < 0) continue;
    if (kind == 4) {
      if (f != BL_CNX && f != BL_CNY) {
        gathered_cp = true;  // component terms: after the wait
        continue;
      }
      if (!x->cn_gather) {
        cudaError_t st = cudaSuccess;
        x->cn_gather = dalloc<double>(x, 8L * x->s.nel, st);
        if (st != cudaSuccess) return BL_FAILURE;
      }
      double* g = x->cn_gather + (f == BL_CNY ? 4L * x->s.nel : 0);
      k_cngather<<<(x->s.nel + 255) / 256, 256, 0, x->stream>>>(
          x->F.ielnd, f == BL_CNX ? x->F.ndx : x->F.ndy, x->s.nel, reinterpret_cast<d4*>(g));
      cudaMemcpyAsync(x->host[f], g, n * sizeof(double), cudaMemcpyDeviceToHost, x->stream);
    } else {
      cudaMemcpyAsync(x->host[f], dev_ptr(x, f), n * sizeof(double), cudaMemcpyDeviceToHost,
                      x->stream);
    }
  }
  cudaError_t r = cudaStreamSynchronize(x->stream);
  if (r == cudaSuccess) r = cudaGetLastError();
  if (r != cudaSuccess) return BL_FAILURE;
  // component iso terms: the element terms gathered to components
  if (gathered_cp) {
    std::vector<double> el(x->s.nel);
    const int* imxel = static_cast<const int*>(x->host[BL_IMXEL]);
    const int* imxfcp = static_cast<const int*>(x->host[BL_IMXFCP]);
    const int* imxncp = static_cast<const int*>(x->host[BL_IMXNCP]);
    for (int k = 0; k < nids; k++) {
      const int f = ids[k];
      if (!x->host[f] || (f != BL_CPA1 && f != BL_CPA3 && f != BL_CPB1 && f != BL_CPB3)) continue;
      int kind;
      field_count(x, f, kind);
      if (kind != 4) continue;
      const double* src = f == BL_CPA1 ? x->F.a1 : f == BL_CPA3 ? x->F.a3 : f == BL_CPB1 ? x->F.b1 : x->F.b3;
      r = cudaMemcpy(el.data(), src, sizeof(double) * x->s.nel, cudaMemcpyDeviceToHost);
      if (r != cudaSuccess) return BL_FAILURE;
      double* h = static_cast<double*>(x->host[f]);
      for (int m = 0; m < x->s.nmx; m++)
        for (int c = 0; c < imxncp[m]; c++) h[imxfcp[m] - 1 + c] = el[imxel[m] - 1];
    }
  }
  if (x->ninst > 0)
    for (int k = 0; k < nids; k++) {
      int kind;
      field_count(x, ids[k], kind);
      if (kind >= 0 && x->host[ids[k]]) batch_copy(x, ids[k], true);
    }
  return BL_SUCCESS;
}

int bl_sync_to_device(bl_ctx* x, int id) {
  if (!x) return BL_FAILURE;
  if (id == 0) {
    for (int k : kStateIds) {
      int rc = bl_sync_to_device(x, k);
      if (rc != BL_SUCCESS) return rc;
    }
    return BL_SUCCESS;
  }
  if (id < 1 || id > BL_NID || !x->host[id]) return BL_SUCCESS;
  int kind;
  size_t n = field_count(x, id, kind);
  if (kind < 0 || kind == 4) return BL_SUCCESS;
  void* d = dev_ptr(x, id);
  if (x->ninst > 0) batch_copy(x, id, false);
  cudaError_t r = cudaMemcpy(d, x->host[id], n * sizeof(double), cudaMemcpyHostToDevice);
  if (id == BL_ELCS2 && r == cudaSuccess)  // keep both copies of elcs2 equal
    r = cudaMemcpy(x->cs2_is_v ? x->F.cs2 : x->F.cs2v, x->host[id], n * sizeof(double),
                   cudaMemcpyHostToDevice);
  return r == cudaSuccess ? BL_SUCCESS : BL_FAILURE;
}

int bl_synchronize(bl_ctx* x) {
  if (!x) return BL_FAILURE;
  return (int)cudaStreamSynchronize(x->stream);
}

void* bl_stream(bl_ctx* x) { return x ? (void*)x->stream : nullptr; }

long long bl_kernel_launches(bl_ctx* x) { return x ? x->launches : 0; }

// Struct sizes, so a host binding can check its mirrors of the header.
int bl_abi_sizes(int* out, int n) {
  const int v[5] = {(int)sizeof(bl_sizes), (int)sizeof(bl_config), (int)sizeof(bl_timestep),
                    (int)sizeof(bl_error), (int)sizeof(bl_step_record)};
  for (int i = 0; i < n && i < 5; i++) out[i] = v[i];
  return 5;
}

}  // extern "C"

// ------------------------------------------------------------------ batches
// Several independent meshes (each one control file's problem) advanced
// together: one kernel per phase over all of them, each mesh with its own
// step header (dt, time, end test, errors).  The host arrays of the meshes
// are concatenated into one disconnected mesh with node, element, region,
// material, component and mixed-cell numbers offset per mesh.

namespace {

enum { kLayNone = 0, kLayEl, kLayCn, kLayNd, kLayEl4, kLayCp, kLayCp4, kLayMx };
enum { kOffNone = 0, kOffNode, kOffEl, kOffReg, kOffMat, kOffCp };
struct FieldLayout {
  int layout, off, is_int;
};

// How a dataAPI field concatenates: per element, per corner, per node, 4
// per element, per component (1 or 4) or per mixed cell, and the numbers
// its values hold.
FieldLayout field_layout(int id) {
  switch (id) {
    case BL_ELDENSITY: case BL_ELENERGY: case BL_ELPRESSURE: case BL_ELCS2: case BL_ELVOLUME:
    case BL_A1: case BL_A2: case BL_A3: case BL_B1: case BL_B2: case BL_B3: case BL_ELVISC:
    case BL_ELMASS:
      return {kLayEl, kOffNone, 0};
    case BL_CNWT: case BL_CNX: case BL_CNY: case BL_CNVISCX: case BL_CNVISCY: case BL_CNMASS:
    case BL_SPMASS:
      return {kLayCn, kOffNone, 0};
    case BL_NDX: case BL_NDY: case BL_NDU: case BL_NDV:
      return {kLayNd, kOffNone, 0};
    case BL_INDTYPE:
      return {kLayNd, kOffReg, 1};  // interior nodes hold their region, boundary ones -bc
    case BL_IELSORT1: case BL_IELSORT2:
      return {kLayEl, kOffEl, 1};
    case BL_IELND:
      return {kLayEl4, kOffNode, 1};
    case BL_IELEL:
      return {kLayEl4, kOffEl, 1};
    case BL_IELFC:
      return {kLayEl4, kOffNone, 1};
    case BL_IELMAT:
      return {kLayEl, kOffMat, 1};
    case BL_IELREG:
      return {kLayEl, kOffReg, 1};
    case BL_CPDENSITY: case BL_CPENERGY: case BL_CPPRESSURE: case BL_CPCS2: case BL_CPVOLUME:
    case BL_FRVOLUME: case BL_CPMASS: case BL_FRMASS: case BL_CPVISC: case BL_CPA1:
    case BL_CPA3: case BL_CPB1: case BL_CPB3:
      return {kLayCp, kOffNone, 0};
    case BL_CPVISCX: case BL_CPVISCY:
      return {kLayCp4, kOffNone, 0};
    case BL_ICPMAT:
      return {kLayCp, kOffMat, 1};
    case BL_ICPNEXT: case BL_ICPPREV:
      return {kLayCp, kOffCp, 1};
    case BL_IMXEL:
      return {kLayMx, kOffEl, 1};
    case BL_IMXFCP:
      return {kLayMx, kOffCp, 1};
    case BL_IMXNCP:
      return {kLayMx, kOffNone, 1};
    default:
      return {kLayNone, kOffNone, 0};
  }
}

size_t layout_count(int layout, const bl_sizes& s) {
  switch (layout) {
    case kLayEl: return (size_t)s.nel;
    case kLayNd: return (size_t)s.nnd;
    case kLayCp: return (size_t)s.ncp;
    case kLayCp4: return 4 * (size_t)s.ncp;
    case kLayMx: return (size_t)s.nmx;
    default: return 4 * (size_t)s.nel;
  }
}

bool same_shared(const bl_config& a, const bl_config& b) {
  return a.cvisc1 == b.cvisc1 && a.cvisc2 == b.cvisc2 && a.cfl_sf == b.cfl_sf &&
         a.div_sf == b.div_sf && a.ztq == b.ztq && a.zhg == b.zhg && a.zsp == b.zsp &&
         a.zcut == b.zcut && a.zerocut == b.zerocut && a.dencut == b.dencut &&
         a.accut == b.accut && a.ccut == b.ccut && a.pcut == b.pcut &&
         a.ale_zexist == b.ale_zexist && a.ale_zon == b.ale_zon && a.ale_zeul == b.ale_zeul &&
         a.ale_adv_type == b.ale_adv_type && a.ale_mintime == b.ale_mintime &&
         a.ale_maxtime == b.ale_maxtime && a.ale_sf == b.ale_sf;
}

// Copies mesh i's part of field id between the concatenated host array and
// the mesh's own registered array (to_mesh: concatenated -> mesh).
void batch_copy(bl_ctx* x, int id, bool to_mesh) {
  const FieldLayout L = field_layout(id);
  if (L.layout == kLayNone || L.is_int || !x->host[id]) return;
  char* all = static_cast<char*>(x->host[id]);
  const std::vector<int>& off = L.layout == kLayNd ? x->nd_off
                                : (L.layout == kLayCp || L.layout == kLayCp4) ? x->cp_off
                                : L.layout == kLayMx ? x->mx_off : x->el_off;
  const size_t per = (L.layout == kLayCn || L.layout == kLayEl4 || L.layout == kLayCp4) ? 4 : 1;
  for (int i = 0; i < x->ninst; i++) {
    void* mine = x->inst_dh[i][id];
    const size_t b = (size_t)off[i] * per, n = (size_t)(off[i + 1] - off[i]) * per;
    if (!mine || n == 0) continue;
    if (to_mesh) std::memcpy(mine, all + 8 * b, 8 * n);
    else std::memcpy(all + 8 * b, mine, 8 * n);
  }
}

void fill_ts_batch(const bl_ctx* x, int i, const DevStep& S, bl_timestep* ts) {
  ts->nstep = S.nstep;
  ts->dt = S.dt;
  ts->time = S.time;
  ts->idtel = S.idtel;
  std::memset(ts->sdt, 0, sizeof ts->sdt);
  std::memcpy(ts->sdt, kSdt[S.sdt < 0 || S.sdt > 4 ? 0 : S.sdt], 8);
  std::memset(ts->mdt, 0, sizeof ts->mdt);
  const int nel_i = x->el_off[i + 1] - x->el_off[i];
  if (S.idtel > 0 && S.idtel <= nel_i) {
    int ii = x->ielmat_h[x->el_off[i] + S.idtel - 1];
    if (ii > 0) {
      ii -= x->mat_off[i];
      ts->imdt = ii;
      std::snprintf(ts->mdt, sizeof ts->mdt, "%10d", ii);
    } else {
      ts->imdt = 0;
      std::memcpy(ts->mdt, "     MIXED", 10);
    }
  } else {
    ts->imdt = -1;
    std::memcpy(ts->mdt, "   UNKNOWN", 10);
  }
  ts->zcorrector = 1;
  ts->dts = ts->dt;
}

}  // namespace

extern "C" {

int bl_init_batch(bl_ctx** out, int ninst, const bl_sizes* sizes, const bl_config* configs,
                  void* const* const* dh, int fp_mode, bl_error* error) {
  set_err(error, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (!out || ninst < 1 || !sizes || !configs || !dh) {
    set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_init_batch: bad argument");
    return BL_FAILURE;
  }
  *out = nullptr;
  const bl_config& c0 = configs[0];
  std::vector<int> el_off(ninst + 1, 0), nd_off(ninst + 1, 0), reg_off(ninst + 1, 0),
      mat_off(ninst + 1, 0), cp_off(ninst + 1, 0), mx_off(ninst + 1, 0);
  for (int i = 0; i < ninst; i++) {
    const bl_sizes& s = sizes[i];
    char msg[BL_SLEN + 1];
    if (!dh[i] || s.nel < 1 || s.nnd < 4 || s.nreg < 1 || s.nreg > BL_MAXREG || s.nmat < 1 ||
        s.nmat > BL_MAXMAT) {
      std::snprintf(msg, sizeof msg, "ERROR: bl_init_batch: mesh %d: sizes out of range", i + 1);
      set_err(error, BL_FAILURE, BL_HALT_ALL, msg);
      return BL_FAILURE;
    }
    if (s.ncp < 0 || s.nmx < 0 || (s.ncp > 0) != (s.nmx > 0)) {
      std::snprintf(msg, sizeof msg, "ERROR: bl_init_batch: mesh %d: mixed-cell sizes", i + 1);
      set_err(error, BL_FAILURE, BL_HALT_ALL, msg);
      return BL_FAILURE;
    }
    if (!same_shared(configs[i], c0)) {
      std::snprintf(msg, sizeof msg,
                    "ERROR: bl_init_batch: mesh %d: hydro, cut-off or ALE settings differ", i + 1);
      set_err(error, BL_FAILURE, BL_HALT_ALL, msg);
      return BL_FAILURE;
    }
    if ((long long)el_off[i] + s.nel > 0x7fffffff || (long long)nd_off[i] + s.nnd > 0x7fffffff ||
        (long long)cp_off[i] + s.ncp > 0x7fffffff) {
      set_err(error, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_init_batch: batch too large");
      return BL_FAILURE;
    }
    el_off[i + 1] = el_off[i] + s.nel;
    nd_off[i + 1] = nd_off[i] + s.nnd;
    reg_off[i + 1] = reg_off[i] + s.nreg;
    mat_off[i + 1] = mat_off[i] + s.nmat;
    cp_off[i + 1] = cp_off[i] + s.ncp;
    mx_off[i + 1] = mx_off[i] + s.nmx;
  }
  bl_sizes S{};
  S.nel = S.nel1 = S.nel2 = el_off[ninst];
  S.nnd = S.nnd1 = S.nnd2 = nd_off[ninst];
  S.nsz = std::max(S.nel, S.nnd);
  S.nreg = reg_off[ninst];
  S.nmat = mat_off[ninst];
  S.ncp = S.mcp = cp_off[ninst];
  S.nmx = S.mmx = mx_off[ninst];
  // the concatenated host arrays
  std::vector<std::vector<char>> store(BL_NID + 1);
  std::vector<void*> cdh(BL_NID + 1, nullptr);
  for (int id = 1; id <= BL_NID; id++) {
    const FieldLayout L = field_layout(id);
    if (L.layout == kLayNone) continue;
    // a field is registered by every mesh that has entries of it (a mesh
    // without mixed cells need not register the component fields)
    int have = 0, need = 0;
    for (int i = 0; i < ninst; i++) {
      const bool some = layout_count(L.layout, sizes[i]) > 0;
      need += some;
      have += some && dh[i][id] != nullptr;
    }
    if (have == 0) continue;
    if (have != need) {
      char msg[BL_SLEN + 1];
      std::snprintf(msg, sizeof msg, "ERROR: bl_init_batch: field %d registered for some meshes only",
                    id);
      set_err(error, BL_FAILURE, BL_HALT_ALL, msg);
      return BL_FAILURE;
    }
    const size_t esz = L.is_int ? 4 : 8;
    store[id].resize(esz * layout_count(L.layout, S));
    size_t at = 0;
    for (int i = 0; i < ninst; i++) {
      const size_t n = layout_count(L.layout, sizes[i]);
      if (n == 0) continue;
      std::memcpy(store[id].data() + esz * at, dh[i][id], esz * n);
      if (L.is_int && L.off != kOffNone) {
        int* v = reinterpret_cast<int*>(store[id].data()) + at;
        const int add = L.off == kOffNode ? nd_off[i] : L.off == kOffEl ? el_off[i]
                      : L.off == kOffReg ? reg_off[i] : L.off == kOffCp ? cp_off[i] : mat_off[i];
        for (size_t k = 0; k < n; k++) {
          if (L.off == kOffNode || L.off == kOffEl || v[k] > 0) v[k] += add;
          else if (id == BL_IELMAT && v[k] < 0) v[k] -= mx_off[i];  // -(mixed cell)
        }
      }
      at += n;
    }
    cdh[id] = store[id].data();
  }
  // region and material tables: mesh after mesh; material 0 (void) once
  Tables T;
  T.et.push_back(c0.eos_type[0]);
  for (int k = 0; k < BL_NEOSPARAM; k++) T.ep.push_back(c0.eos_param[0][k]);
  for (int i = 0; i < ninst; i++) {
    const bl_config& c = configs[i];
    for (int r = 0; r < sizes[i].nreg; r++) {
      T.kap.push_back(c.kappareg[r]);
      T.pm.push_back(c.pmeritreg[r]);
      T.zd.push_back(c.zdtnotreg[r]);
      T.zm.push_back(c.zmidlength[r]);
    }
    for (int m = 1; m <= sizes[i].nmat; m++) {
      T.et.push_back(c.eos_type[m]);
      for (int k = 0; k < BL_NEOSPARAM; k++) T.ep.push_back(c.eos_param[m][k]);
    }
  }
  bl_config C = c0;
  int rc = init_impl(out, &S, &C, cdh.data(), fp_mode, error, &T);
  if (rc != BL_SUCCESS) return rc;
  bl_ctx* x = *out;
  x->bstore = std::move(store);  // the context's host fields point into these
  x->ninst = ninst;
  x->el_off = el_off;
  x->nd_off = nd_off;
  x->mat_off = mat_off;
  x->cp_off = cp_off;
  x->mx_off = mx_off;
  x->inst_dh.resize(ninst);
  for (int i = 0; i < ninst; i++) x->inst_dh[i].assign(dh[i], dh[i] + BL_NID + 1);
  // per-mesh controls and ownership tables
  std::vector<bl::DevInst> inst(ninst);
  std::vector<int> elinst(S.nel), ndinst(S.nnd), blkinst;
  int nblk = 0;
  for (int i = 0; i < ninst; i++) {
    const bl_config& c = configs[i];
    bl::DevInst& I = inst[i];
    I.dt_g = c.dt_g;
    I.dt_min = c.dt_min;
    I.dt_max = c.dt_max;
    I.dt_initial = c.dt_initial;
    I.time_end = c.time_end;
    I.el_begin = el_off[i];
    I.el_end = el_off[i + 1];
    I.blk_begin = nblk;
    nblk += x->L.getdt_blocks(sizes[i].nel);
    I.blk_end = nblk;
    for (int k = el_off[i]; k < el_off[i + 1]; k++) elinst[k] = i;
    for (int k = nd_off[i]; k < nd_off[i + 1]; k++) ndinst[k] = i;
    blkinst.insert(blkinst.end(), I.blk_end - I.blk_begin, i);
  }
  cudaError_t st = cudaSuccess;
  bl::DevFields& F = x->F;
  F.steps = dalloc<DevStep>(x, ninst, st);
  bl::DevInst* d_inst = dalloc<bl::DevInst>(x, ninst, st);
  int* d_el = dalloc<int>(x, S.nel, st);
  int* d_nd = dalloc<int>(x, S.nnd, st);
  int* d_bk = dalloc<int>(x, nblk, st);
  double* d_rv = dalloc<double>(x, 2L * nblk, st);
  int* d_ri = dalloc<int>(x, 2L * nblk, st);
  if (st != cudaSuccess || cudaMallocHost(&x->hsteps, sizeof(DevStep) * ninst) != cudaSuccess) {
    bl_finalize(x);
    *out = nullptr;
    return cuda_fail(error, st == cudaSuccess ? cudaErrorMemoryAllocation : st, "bl_init_batch");
  }
  up(x, d_inst, inst.data(), ninst);
  x->inst_h = inst;
  up(x, d_el, elinst.data(), S.nel);
  up(x, d_nd, ndinst.data(), S.nnd);
  up(x, d_bk, blkinst.data(), nblk);
  F.inst = d_inst;
  F.elinst = d_el;
  F.ndinst = d_nd;
  F.blkinst = d_bk;
  F.red_v = d_rv;  // partials of every mesh's blocks
  F.red_i = d_ri;
  F.ninst = ninst;
  F.nblk_batch = nblk;
  F.nd_block = 256;
  cudaError_t r = cudaStreamSynchronize(x->stream);
  if (r != cudaSuccess) {
    bl_finalize(x);
    *out = nullptr;
    return cuda_fail(error, r, "bl_init_batch");
  }
  return BL_SUCCESS;
}

int bl_run_batch(bl_ctx* x, bl_timestep* ts, int max_steps, int* status, int* nsteps,
                 bl_error* e) {
  set_err(e, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (nsteps) *nsteps = 0;
  if (!x || !ts || max_steps < 0 || x->ninst < 1) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_run_batch: bad argument (or not a batch)");
    return BL_FAILURE;
  }
  if (x->c.ale_zexist && x->c.ale_adv_type != 1) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_run_batch: only adv_type 1 runs on the device");
    return BL_FAILURE;
  }
  const int n = x->ninst;
  for (int i = 0; i < n; i++) {
    DevStep& h = x->hsteps[i];
    std::memset(&h, 0, sizeof h);
    h.time = ts[i].time;
    h.dt = ts[i].dt;
    h.dts = ts[i].dts;
    h.rdt = 1.0 / ts[i].dt;
    h.nstep = ts[i].nstep;
    h.idtel = ts[i].idtel;
    h.run_mode = 1;
    // a mesh already at its end time does not advance (the others do)
    if (ts[i].time >= x->inst_h[i].time_end) h.stop_next = 1;
  }
  cudaMemcpyAsync(x->F.steps, x->hsteps, sizeof(DevStep) * n, cudaMemcpyHostToDevice, x->stream);
  if (max_steps == 0) return bl_synchronize(x) == 0 ? BL_SUCCESS : BL_FAILURE;
  const bool with_ale = x->c.ale_zexist != 0;
  const int G = x->b_graph_steps;  // steps per graph launch
  cudaError_t r;
  bl::DevFields F = x->F;
  F.hist = nullptr;
  bl::DevCfg C = x->C;
  C.max_records = 0;
  auto queue_step = [&]() {
    x->L.getdt_b(F, C, x->stream);
    x->L.lag_force_b(F, C, x->stream);
    x->L.lag_accel_b(F, C, x->stream);
    x->L.lag_state_b(F, C, x->stream);
    x->L.mix_closure_b(F, C, x->stream);
    if (with_ale) x->L.ale_b(F, C, x->stream);
  };
  if (!x->bexec || x->b_ale != with_ale || x->b_gsteps != G || x->b_ndblock != F.nd_block) {
    if (x->bexec) cudaGraphExecDestroy(x->bexec);
    x->bexec = nullptr;
    cudaGraph_t g;
    r = cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal);
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run_batch capture");
    for (int k = 0; k < G; k++) queue_step();
    r = cudaStreamEndCapture(x->stream, &g);
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run_batch capture");
    r = cudaGraphInstantiate(&x->bexec, g, 0);
    cudaGraphDestroy(g);
    if (r != cudaSuccess) {
      x->bexec = nullptr;
      return cuda_fail(e, r, "bl_run_batch instantiate");
    }
    x->b_ale = with_ale;
    x->b_gsteps = G;
    x->b_ndblock = F.nd_block;
  }
  const int per_step = x->L.getdt_launches(x->C) + bl::launches_lagstep(x->F) + (with_ale ? bl::kLaunchesAle : 0);
  int done = 0;
  while (done < max_steps) {
    const int k = std::min(G, max_steps - done);
    if (k == G) {
      r = cudaGraphLaunch(x->bexec, x->stream);
      if (r != cudaSuccess) return cuda_fail(e, r, "bl_run_batch launch");
    } else {
      for (int j = 0; j < k; j++) queue_step();
    }
    x->launches += (long long)k * per_step;
    done += k;
    cudaMemcpyAsync(x->hsteps, x->F.steps, sizeof(DevStep) * n, cudaMemcpyDeviceToHost, x->stream);
    r = cudaStreamSynchronize(x->stream);
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run_batch");
    r = cudaGetLastError();
    if (r != cudaSuccess) return cuda_fail(e, r, "bl_run_batch");
    int active = 0;
    for (int i = 0; i < n; i++) {
      const DevStep& S = x->hsteps[i];
      if (!(S.halted || S.stop_next || S.err_code || S.negvol_pred || S.negvol_corr ||
            S.negvol_ale))
        active++;
    }
    if (active == 0) break;
  }
  if (nsteps) *nsteps = done;
  int first_bad = -1;
  for (int i = 0; i < n; i++) {
    const DevStep& S = x->hsteps[i];
    fill_ts_batch(x, i, S, ts + i);
    int code = 0;
    if (S.err_code == 1 || S.err_code == 2) code = BL_FAILURE;
    else if (S.negvol_pred) code = -S.negvol_pred;
    else if (S.negvol_corr) code = -S.negvol_corr;
    else if (S.negvol_ale) code = -S.negvol_ale;
    if (status) status[i] = code;
    if (code != 0 && first_bad < 0) first_bad = i;
  }
  x->cs2_is_v = false;
  if (first_bad >= 0) {
    const DevStep& S = x->hsteps[first_bad];
    char msg[BL_SLEN + 1];
    std::snprintf(msg, sizeof msg, "ERROR: mesh %d: %s", first_bad + 1,
                  S.err_code == 1 ? "negative CFL condition in hydro_dr_getdt"
                  : S.err_code == 2 ? "dt < dt_min"
                                    : "negative volume in geometry_dr_getgeometry");
    set_err(e, BL_FAILURE, S.err_code == 2 ? BL_HALT_ALL : BL_HALT_SINGLE, msg);
    return BL_FAILURE;
  }
  return BL_SUCCESS;
}

int bl_batch_size(bl_ctx* x) { return x ? x->ninst : 0; }

const float* bl_mlp_device_image(bl_mlp* m);  // bl_mlp.cu

int bl_set_closure(bl_ctx* x, bl_mlp* net, const float* norm, int on, bl_error* e) {
  set_err(e, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (!x || on < 0 || on > 2 || (on && (!net || !norm))) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_set_closure: bad argument");
    return BL_FAILURE;
  }
  bl::DevFields& F = x->F;
  if (on) {
    cudaError_t st = cudaSuccess;
    if (!F.mxv0) F.mxv0 = dalloc<double>(x, std::max(1, x->s.nmx), st);
    if (!F.mlp_norm) F.mlp_norm = dalloc<float>(x, 2 * BL_MLP_IN + 2, st);
    if (!F.mlp_count) F.mlp_count = dalloc<unsigned long long>(x, 2, st);
    if (!F.mlp_img) F.mlp_img = dalloc<float>(x, bl::mlp::kImgN, st);
    if (st != cudaSuccess || x->L.mix_prepare() != 0) return cuda_fail(e, cudaErrorMemoryAllocation, "bl_set_closure");
    cudaMemcpyAsync(const_cast<float*>(F.mlp_norm), norm, (2 * BL_MLP_IN + 2) * sizeof(float),
                    cudaMemcpyHostToDevice, x->stream);
    // the network as it is now (training it further changes nothing here)
    cudaDeviceSynchronize();
    cudaMemcpyAsync(F.mlp_img, bl_mlp_device_image(net), bl::mlp::kImgN * sizeof(float),
                    cudaMemcpyDeviceToDevice, x->stream);
  }
  F.closure = on;
  // the device loops' graphs hold the old arguments
  if (x->gexec) cudaGraphExecDestroy(x->gexec);
  x->gexec = nullptr;
  if (x->bexec) cudaGraphExecDestroy(x->bexec);
  x->bexec = nullptr;
  return cudaStreamSynchronize(x->stream) == cudaSuccess ? BL_SUCCESS : BL_FAILURE;
}

int bl_closure_stats(bl_ctx* x, unsigned long long* cells, unsigned long long* rejected) {
  if (!x) return BL_FAILURE;
  unsigned long long h[2] = {0, 0};
  if (x->F.mlp_count &&
      cudaMemcpy(h, x->F.mlp_count, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess)
    return BL_FAILURE;
  if (cells) *cells = h[0];
  if (rejected) *rejected = h[1];
  return BL_SUCCESS;
}

// The batch's autotuner: steps per graph G in {8, 16, 32} and the node
// kernels' block size in {128, 256, 512}, each candidate timed (CUDA
// events on the context's stream, host polling included) over the same 32
// steps from the state held by the meshes' registered host arrays, after one
// untimed graph that instantiates it; the state is uploaded again before
// every run and after the last.
int bl_autotune_batch(bl_ctx* x, const bl_timestep* ts, int* graph_steps, int* node_block,
                      double* ms_per_step, int n_ms, bl_error* e) {
  set_err(e, BL_SUCCESS, BL_HALT_SINGLE, "");
  if (!x || !ts || x->ninst < 1) {
    set_err(e, BL_FAILURE, BL_HALT_ALL, "ERROR: bl_autotune_batch: bad argument (or not a batch)");
    return BL_FAILURE;
  }
  static const int kG[3] = {8, 16, 32}, kB[3] = {128, 256, 512};
  const int n = x->ninst;
  std::vector<bl_timestep> tsc(n);
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
    return cuda_fail(e, cudaErrorMemoryAllocation, "bl_autotune_batch");
  double best = 1e300;
  int bg = 16, bb = 256, k = 0, rc = BL_SUCCESS;
  for (int gi = 0; gi < 3 && rc == BL_SUCCESS; gi++)
    for (int bi = 0; bi < 3 && rc == BL_SUCCESS; bi++, k++) {
      x->b_graph_steps = kG[gi];
      x->F.nd_block = kB[bi];
      float t = 0.0f;
      for (int pass = 0; pass < 2 && rc == BL_SUCCESS; pass++) {
        rc = bl_sync_to_device(x, 0);
        if (rc != BL_SUCCESS) break;
        tsc.assign(ts, ts + n);
        int ns = 0;
        if (pass == 1) cudaEventRecord(a, x->stream);
        rc = bl_run_batch(x, tsc.data(), pass == 0 ? kG[gi] : 32, nullptr, &ns, e);
        if (pass == 1) {
          cudaEventRecord(b, x->stream);
          cudaEventSynchronize(b);
          cudaEventElapsedTime(&t, a, b);
          t /= (float)std::max(1, ns);
        }
      }
      if (rc != BL_SUCCESS) break;
      if (ms_per_step && k < n_ms) ms_per_step[k] = t;
      if (t < best) {
        best = t;
        bg = kG[gi];
        bb = kB[bi];
      }
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  x->b_graph_steps = bg;
  x->F.nd_block = bb;
  if (rc == BL_SUCCESS) rc = bl_sync_to_device(x, 0);
  if (graph_steps) *graph_steps = bg;
  if (node_block) *node_block = bb;
  return rc;
}

}  // extern "C"
