// bl_kernels.h -- launch functions of the kernel translation unit.
//
// bl_kernels.cu is compiled three times: as namespace bl::exact with
// --fmad=false (bit-reproducible against a -ffp-contract=off CPU build), as
// bl::fast with --fmad=true, and as bl::mixed, the fast build with the
// limiter and edge-viscosity arithmetic in FP32 (BL_MIXED, bl_lreal.cuh).  The C-ABI layer picks one
// table per context (bl_init's fp_mode).
#pragma once
#include <cuda_runtime.h>

#include "bl_device.cuh"

namespace bl {

#define BL_DECLARE_LAUNCHERS(NS)                                                   \
  namespace NS {                                                                   \
  int getdt_blocks(int nel);                                                       \
  int getdt_grid(int nel);                                                         \
  void launch_getdt(const DevFields& F, const DevCfg& C, cudaStream_t s);          \
  void launch_lag_force(const DevFields& F, const DevCfg& C, cudaStream_t s);      \
  void launch_lag_accel(const DevFields& F, const DevCfg& C, cudaStream_t s);      \
  void launch_lag_state(const DevFields& F, const DevCfg& C, cudaStream_t s);      \
  void launch_ale(const DevFields& F, const DevCfg& C, cudaStream_t s);            \
  void launch_getdt_batch(const DevFields& F, const DevCfg& C, cudaStream_t s);    \
  void launch_lag_force_batch(const DevFields& F, const DevCfg& C, cudaStream_t s);\
  void launch_lag_accel_batch(const DevFields& F, const DevCfg& C, cudaStream_t s);\
  void launch_lag_state_batch(const DevFields& F, const DevCfg& C, cudaStream_t s);\
  void launch_ale_batch(const DevFields& F, const DevCfg& C, cudaStream_t s);      \
  int prepare_mix_closure();                                                       \
  void launch_mix_closure(const DevFields& F, const DevCfg& C, cudaStream_t s);    \
  void launch_mix_closure_batch(const DevFields& F, const DevCfg& C, cudaStream_t s);\
  int getdt_launches(const DevCfg& C);                                             \
  }

BL_DECLARE_LAUNCHERS(fast)
BL_DECLARE_LAUNCHERS(exact)
BL_DECLARE_LAUNCHERS(mixed)

struct Launchers {
  int (*getdt_blocks)(int);  // k_getdt blocks of one mesh in a batch
  int (*getdt_grid)(int);    // k_getdt grid (and partials) of a single mesh
  void (*getdt)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*lag_force)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*lag_accel)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*lag_state)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*ale)(const DevFields&, const DevCfg&, cudaStream_t);
  // the same over a batch of meshes (per-mesh step headers)
  void (*getdt_b)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*lag_force_b)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*lag_accel_b)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*lag_state_b)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*ale_b)(const DevFields&, const DevCfg&, cudaStream_t);
  // the learned mixed-cell closure (after lag_state; no-op when off)
  int (*mix_prepare)();
  void (*mix_closure)(const DevFields&, const DevCfg&, cudaStream_t);
  void (*mix_closure_b)(const DevFields&, const DevCfg&, cudaStream_t);
  // kernels one getdt launcher call launches (for bl_kernel_launches)
  int (*getdt_launches)(const DevCfg&);
};

// Kernels launched by one call of each launcher (for bl_kernel_launches;
// getdt's: Launchers::getdt_launches).
constexpr int kLaunchesLagstep = 3;
constexpr int kLaunchesAle = 4;
// the lagstep launcher's count with the learned closure in it
inline int launches_lagstep(const DevFields& F) {
  return kLaunchesLagstep + (F.closure && F.nmx > 0 ? 1 : 0);
}

}  // namespace bl
