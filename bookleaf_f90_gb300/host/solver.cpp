// solver.cpp -- the reference's solver entry points over the C-ABI:
//   inf_solver_getdt   (inf_solver_getdt.f90:35-70)
//   inf_solver_lagstep (inf_solver_lagstep.f90:44-78)
//   inf_solver_alestep (inf_solver_alestep.f90:39-74)
// and the loop of inf_control_solver (inf_control_solver.f90:53-69).
#include "blh.hpp"

namespace blh {

Solver::Solver(Problem& p, int fp_mode) : p_(p) {
  tab_ = p.pointer_table();
  const int ierr = bl_init(&ctx_, &p.sizes, &p.config, tab_.data(), fp_mode, &err_);
  if (ierr != BL_SUCCESS) throw SolverError(ierr, err_.iout, err_.serr);
}

Solver::~Solver() {
  if (ctx_) bl_finalize(ctx_);
}

int Solver::inf_solver_getdt(bl_timestep& ts) { return bl_getdt(ctx_, &ts, &err_); }
int Solver::inf_solver_lagstep(bl_timestep& ts) { return bl_lagstep(ctx_, &ts, &err_); }
int Solver::inf_solver_alestep(bl_timestep& ts) { return bl_alestep(ctx_, &ts, &err_); }

int Solver::step(bl_timestep& ts) {
  int ierr = inf_solver_getdt(ts);
  if (ierr != BL_SUCCESS) return ierr;
  ierr = inf_solver_lagstep(ts);
  if (ierr != BL_SUCCESS) return ierr;
  return inf_solver_alestep(ts);
}

int Solver::run(bl_timestep& ts, int max_steps, int* nsteps) {
  return bl_run(ctx_, &ts, max_steps, nullptr, nsteps, &err_);
}

void Solver::sync_to_host(int id) {
  if (bl_sync_to_host(ctx_, id) != BL_SUCCESS) throw SolverError(BL_FAILURE, BL_HALT_ALL, "bl_sync_to_host failed");
}

void Solver::sync_to_device(int id) {
  if (bl_sync_to_device(ctx_, id) != BL_SUCCESS)
    throw SolverError(BL_FAILURE, BL_HALT_ALL, "bl_sync_to_device failed");
}

std::vector<FlagTotals> Solver::shortprint(bool by_material) {
  const int n = by_material ? p_.sizes.nmat : p_.sizes.nreg;
  std::vector<double> out((size_t)n * BL_SP_NQ);
  if (bl_shortprint(ctx_, by_material ? 1 : 0, out.data(), n, &err_) != BL_SUCCESS)
    throw SolverError(err_.ierr, err_.iout, err_.serr);
  std::vector<FlagTotals> t(n);
  for (int i = 0; i < n; i++) {
    const double* r = &out[(size_t)i * BL_SP_NQ];
    t[i].vol = r[0];
    t[i].mass = r[1];
    t[i].ie = r[2];
    t[i].ke = r[3];
    t[i].pressure = r[4];
    t[i].pmn = r[5];
    t[i].pmx = r[6];
    t[i].density = r[7];
    t[i].dmn = r[8];
    t[i].dmx = r[9];
  }
  return t;
}

void Solver::check_sod(double time, double& l1_density, double& l1_energy) {
  if (bl_check_sod(ctx_, time, &l1_density, &l1_energy, &err_) != BL_SUCCESS)
    throw SolverError(err_.ierr, err_.iout, err_.serr);
}

}  // namespace blh
