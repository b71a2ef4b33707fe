// blh.hpp -- C++ host side of the GB300 hydro path: the reference's set-up
// sequence (control file, mesh, connectivity, node types, initial state)
// and its solver entry points, over the C-ABI of include/bookleaf_gb300.h.
//
// Restated from the reference (file:line of each routine at its
// definition):
//   control-file namelists   setup_read.f90, setup_mesh.F90, setup_IC.f90
//   LIN1/LIN2 mesh           setup_mesh.F90:593-1250
//   connectivity             utils_kn_connectivity.f90:30-170
//   node types               init_kn.f90:78-106
//   initial state            setup_IC.f90:268-811, init_kn.f90:32-63,
//                            hydro_kn_init.f90:46-77
//   solver entry points      inf_solver_getdt.f90:35-70,
//                            inf_solver_lagstep.f90:44-78,
//                            inf_solver_alestep.f90:39-74
//   time loop                inf_control_solver.f90:53-69
//
// Every floating-point formula is evaluated in the reference's order with
// IEEE double operations (the build compiles this code with
// -ffp-contract=off), so the state handed to the device equals the one the
// reference's set-up produces.
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/bookleaf_gb300.h"

namespace blh {

// A control file the reference would reject (same messages).
struct DeckError : std::runtime_error {
  explicit DeckError(const std::string& m) : std::runtime_error(m) {}
};

// ---------------------------------------------------------------- namelists

struct Value {
  enum Kind { NONE, STR, BOOL, INT, REAL } kind = NONE;
  std::string s;
  bool b = false;
  long long i = 0;
  double d = 0.0;
  static Value str(const std::string& v) { Value x; x.kind = STR; x.s = v; return x; }
  static Value boolean(bool v) { Value x; x.kind = BOOL; x.b = v; return x; }
  static Value integer(long long v) { Value x; x.kind = INT; x.i = v; return x; }
  static Value real(double v) { Value x; x.kind = REAL; x.d = v; return x; }
  double as_real() const;
  long long as_int() const;
  bool as_bool() const;
  std::string as_str() const;     // upper-cased and stripped for comparisons
};

// One namelist group: name -> scalar, or name -> {1-based index tuple: value}.
struct Entry {
  bool is_array = false;
  Value scalar;
  std::map<std::vector<int>, Value> items;
};

class Namelist {
 public:
  std::map<std::string, Entry> vars;
  bool has(const std::string& name) const;
  Value get_scalar(const std::string& name, const Value& dflt) const;
  // Flat C-order array over `shape` (0-based), filled with dflt and the
  // assigned items.
  std::vector<Value> get_array(const std::string& name, const std::vector<int>& shape,
                               const Value& dflt) const;
};

using Groups = std::map<std::string, Namelist>;

Groups parse_deck(const std::string& text);
bl_config build_config(const Groups& groups, int nreg, int nmat);

// ---------------------------------------------------------------- problem

// A BookLeaf problem on the host: sizes, config, every dataAPI field the
// path uses (element fields nel, corner/face fields as (NCORN,nel) blocks,
// node fields nnd, 1-based integer connectivity) and the timestep.
struct Problem {
  bl_sizes sizes{};
  bl_config config{};
  bl_timestep timestep{};
  std::map<int, std::vector<double>> real;  // dataAPI id -> values
  std::map<int, std::vector<int>> ints;
  // region and material names in indicator order (for the short print)
  std::vector<std::string> region_names, material_names;
  std::array<void*, BL_NID + 1> pointer_table();
  int nel() const { return sizes.nel; }
  int nnd() const { return sizes.nnd; }
};

Problem problem_from_deck(const std::string& text);
std::string read_file(const std::string& path);

// Set-up dump (tests compare it with the Python harness array by array).
void write_setup_dump(const Problem& p, const std::string& path);

// The reference's visualisation dump (io_dr_silo.f90:70-262) as a VTK
// legacy unstructured grid: mesh, materials with volume fractions,
// density, energy, pressure, region, node velocity (io.cpp).
void write_vtk(const Problem& p, const std::string& path);

// hydro_kn_calc_shortprint (hydro_kn_print.F90:52-101) per region or
// material flag: volume, mass, internal and kinetic energy, mass-weighted
// pressure, pressure and density extremes (and the averages of
// hydro_kn_average_shortprint when computed on the device).
struct FlagTotals {
  double vol = 0, mass = 0, ie = 0, ke = 0, pressure = 0;
  double pmn = 0, pmx = 0, dmn = 0, dmx = 0;
  double density = 0;
};

// ---------------------------------------------------------------- solver

// Error carried out of a failed entry point: error_t{ierr,iout,serr}.
struct SolverError : std::runtime_error {
  int ierr, iout;
  SolverError(int e, int o, const std::string& m) : std::runtime_error(m), ierr(e), iout(o) {}
};

// The Fortran host's view of the path: registers the problem's arrays with
// bl_init (like dh(:)) and exposes the three entry points under the
// reference's names; each returns error%ierr and leaves error%iout/serr in
// error().
class Solver {
 public:
  Solver(Problem& p, int fp_mode = BL_FP_FAST);
  ~Solver();
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  int inf_solver_getdt(bl_timestep& ts);
  int inf_solver_lagstep(bl_timestep& ts);
  int inf_solver_alestep(bl_timestep& ts);
  // one cycle of inf_control_solver's loop
  int step(bl_timestep& ts);
  // the whole loop on the device (bl_run); nsteps receives the steps taken
  int run(bl_timestep& ts, int max_steps, int* nsteps);
  void sync_to_host(int id = 0);
  void sync_to_device(int id = 0);
  // diagnostics from the device state (bl_shortprint, bl_check_sod)
  std::vector<FlagTotals> shortprint(bool by_material);
  void check_sod(double time, double& l1_density, double& l1_energy);
  const bl_error& error() const { return err_; }
  bl_ctx* ctx() { return ctx_; }

 private:
  Problem& p_;
  std::array<void*, BL_NID + 1> tab_{};
  bl_ctx* ctx_ = nullptr;
  bl_error err_{};
};

// ---------------------------------------------------------------- reports

// host-side short print of a Problem's fields (elements only), with the
// averages of hydro_kn_average_shortprint
std::vector<FlagTotals> shortprint(const Problem& p, bool by_material);
// the short print (hydro_kn_write_*_shortprint layout) from host tables
std::string format_shortprint(const Problem& p, int nstep, double time);
std::string format_shortprint(const Problem& p, int nstep, double time,
                              const std::vector<FlagTotals>& regions,
                              const std::vector<FlagTotals>& materials);

// check_kn_sod (check_kn_tests.f90:33-111): L1 norms of density and energy
// against the exact Sod solution in the check's geometry (x in [0,100],
// interface at x = 50, gamma 1.4).
void check_sod(const Problem& p, double time, double& l1_density, double& l1_energy);

}  // namespace blh
