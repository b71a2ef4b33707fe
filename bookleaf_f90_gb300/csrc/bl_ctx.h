// bl_ctx.h -- the library context behind the opaque bl_ctx of the C-ABI:
// device mirrors, configuration tables, stream, launchers and the state of
// the device time loop.  Shared by the C-ABI sources of the library.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/bookleaf_gb300.h"
#include "bl_device.cuh"
#include "bl_kernels.h"

struct bl_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bl_sizes s{};
  bl_config c{};
  int fp_mode = BL_FP_FAST;
  void* host[BL_NID + 1] = {};
  bl::DevFields F{};
  bl::DevCfg C{};
  bl::Launchers L{};
  std::vector<void*> bufs;
  // the device arena the arrays are carved from (dalloc)
  char* arena_ptr = nullptr;
  size_t arena_left = 0, arena_next = 0;
  double* cn_gather = nullptr;  // [2][4*nel]: cnx, cny gathered for bl_sync_to_host
  bl::DevStep* hstep = nullptr;  // pinned mirror of F.step
  // true while *hstep equals F.step on the device: set by a completed
  // fetch of the header, cleared whenever work that may change it is queued
  bool hstep_current = false;
  bool cs2_is_v = false;     // elcs2 currently holds cs2 + elvisc (after getdt)
  long long launches = 0;
  // per-call entry points: one cached graph each (getdt, lagstep, alestep)
  // of their kernels and the header download, with the kernel arguments it
  // was captured with
  cudaGraphExec_t call_exec[3] = {nullptr, nullptr, nullptr};
  bl::DevFields call_F[3] = {};
  bl::DevCfg call_C[3] = {};
  // a batch of meshes (bl_init_batch); ninst = 0 for a single mesh
  int ninst = 0;
  std::vector<int> el_off, nd_off, mat_off;    // [ninst+1] first element, node, material
  std::vector<int> cp_off, mx_off;             // [ninst+1] first component, mixed cell
  bl::DevStep* hsteps = nullptr;               // pinned mirror of F.steps
  std::vector<bl::DevInst> inst_h;             // host copy of the per-mesh controls
  std::vector<std::vector<void*>> inst_dh;     // each mesh's registered host arrays
  std::vector<std::vector<char>> bstore;       // the concatenated host arrays, by field
  cudaGraphExec_t bexec = nullptr;             // graph of batch steps
  bool b_ale = false;
  int b_graph_steps = 16;                      // steps per graph (autotuned)
  int b_gsteps = 0, b_ndblock = 0;             // what bexec was captured with
  // bl_run
  cudaGraphExec_t gexec = nullptr;
  int gsteps = 0;
  bool g_ale = false;
  bl::StepRec* g_hist = nullptr;  // history buffer and record limit the
  int g_maxrec = -1;              // graph's kernel arguments were captured with
  int hist_cap = 0;
  std::vector<int> ielmat_h;  // for timestep%mdt
  // diagnostics scratch (bl_shortprint, bl_check_sod), grown on demand
  double* diag = nullptr;
  size_t diag_cap = 0;
};
