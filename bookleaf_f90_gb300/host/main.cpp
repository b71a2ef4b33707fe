// main.cpp -- bookleaf_gb300: runs a BookLeaf control file on the GB300 path,
// the C++ counterpart of the reference's executable for the hot path
// (inf_control_main.f90: init, the solver loop, short prints, validation).
//
//   bookleaf_gb300 [--fp fast|exact|mixed] [--calls] [--max-steps N]
//                  [--print-every N] [--dump-setup FILE] [--dump-final FILE]
//                  [--vtk FILE] [--vtk-setup FILE] CONTROL_FILE
//
// --calls runs the loop of inf_control_solver on the host, one call per
// entry point per step, printing a step line like time_dr_utils.f90:47-50;
// the default runs it on the device (bl_run).  --dump-setup writes the
// initial state and exits without touching a GPU.  --vtk writes the final
// state as the reference's visualisation dump (io_dr_silo.f90, as VTK:
// io.cpp); --vtk-setup writes the initial state so and exits without a
// GPU.  A control file whose
// name contains "sod" is validated with the reference's Sod check
// (check_dr_validate.f90).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "blh.hpp"

namespace {

void usage() {
  std::fprintf(stderr,
               "usage: bookleaf_gb300 [--fp fast|exact|mixed] [--calls] [--max-steps N]\n"
               "                      [--print-every N] [--dump-setup FILE] [--dump-final FILE]\n"
               "                      [--vtk FILE] [--vtk-setup FILE] CONTROL_FILE\n");
}

std::string trimmed(const char* s, size_t n) {
  std::string r(s, strnlen(s, n));
  while (!r.empty() && (r.back() == ' ' || r.back() == '\0')) r.pop_back();
  return r;
}

}  // namespace

int main(int argc, char** argv) {
  int fp = BL_FP_FAST;
  bool calls = false;
  long max_steps = 2147483647L;
  long print_every = 0;
  std::string deck, dump_setup, dump_final, vtk, vtk_setup;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) {
        usage();
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "--fp") {
      const std::string m = next();
      if (m == "fast") fp = BL_FP_FAST;
      else if (m == "exact") fp = BL_FP_EXACT;
      else if (m == "mixed") fp = BL_FP_MIXED;
      else {
        usage();
        return 2;
      }
    } else if (a == "--calls") {
      calls = true;
    } else if (a == "--max-steps") {
      max_steps = std::atol(next().c_str());
    } else if (a == "--print-every") {
      print_every = std::atol(next().c_str());
    } else if (a == "--dump-setup") {
      dump_setup = next();
    } else if (a == "--dump-final") {
      dump_final = next();
    } else if (a == "--vtk") {
      vtk = next();
    } else if (a == "--vtk-setup") {
      vtk_setup = next();
    } else if (!a.empty() && a[0] == '-') {
      usage();
      return 2;
    } else {
      deck = a;
    }
  }
  if (deck.empty()) {
    usage();
    return 2;
  }
  blh::Problem p;
  try {
    p = blh::problem_from_deck(blh::read_file(deck));
  } catch (const blh::DeckError& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  std::printf(" BookLeaf GB300 (%s)\n control file: %s\n nel=%d nnd=%d nreg=%d nmat=%d ncp=%d\n",
              bl_version(), deck.c_str(), p.sizes.nel, p.sizes.nnd, p.sizes.nreg, p.sizes.nmat,
              p.sizes.ncp);
  if (!dump_setup.empty() || !vtk_setup.empty()) {
    if (!dump_setup.empty()) {
      blh::write_setup_dump(p, dump_setup);
      std::printf(" initial state written to %s\n", dump_setup.c_str());
    }
    if (!vtk_setup.empty()) {
      blh::write_vtk(p, vtk_setup);
      std::printf(" initial state dump written to %s\n", vtk_setup.c_str());
    }
    return 0;
  }
  int rc = 0;
  try {
    blh::Solver s(p, fp);
    // short prints from the device state (bl_shortprint): no field copy
    auto print = [&](const bl_timestep& t) {
      std::fputs(blh::format_shortprint(p, t.nstep, t.time, s.shortprint(false), s.shortprint(true))
                     .c_str(),
                 stdout);
    };
    print(p.timestep);
    bl_timestep& ts = p.timestep;
    const auto t0 = std::chrono::steady_clock::now();
    long nsteps = 0;
    int ierr = 0;
    if (calls) {
      while (ts.time < p.config.time_end && nsteps < max_steps) {
        ierr = s.step(ts);
        if (ierr != BL_SUCCESS) break;
        nsteps++;
        if (print_every > 0 && nsteps % print_every == 0) {
          const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
          std::printf(" step=%7d  el=%9d %10s dt=%16.9e  time=%16.9e  grind=%8.1e  timer=%16.9e s\n",
                      ts.nstep, ts.idtel, trimmed(ts.sdt, sizeof ts.sdt).c_str(), ts.dt, ts.time,
                      el * 1e6 / ((double)nsteps * p.sizes.nel), el);
        }
      }
    } else {
      int n = 0;
      ierr = s.run(ts, (int)max_steps, &n);
      nsteps = n;
    }
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (ierr != BL_SUCCESS) {
      std::printf("\n %s\n", trimmed(s.error().serr, sizeof s.error().serr).c_str());
      rc = 1;
    }
    print(ts);
    std::printf("\n %ld steps in %.3f s: %.3e zone-cycles/s, grind %.3e us\n", nsteps, el,
                nsteps * (double)p.sizes.nel / el, el * 1e6 / ((double)nsteps * p.sizes.nel));
    if (deck.find("sod") != std::string::npos) {
      double l1d, l1e;
      s.check_sod(ts.time, l1d, l1e);
      std::printf(" VALIDATION\n  Sod shocktube test case\n   L1 norm. of density: %16.9e\n", l1d);
    }
    if (!dump_final.empty() || !vtk.empty()) s.sync_to_host(0);
    if (!dump_final.empty()) blh::write_setup_dump(p, dump_final);
    if (!vtk.empty()) {
      blh::write_vtk(p, vtk);
      std::printf(" dump written to %s\n", vtk.c_str());
    }
  } catch (const blh::SolverError& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return rc;
}
