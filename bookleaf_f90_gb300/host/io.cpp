// io.cpp -- the reference's visualisation dump (io_dr_silo.f90:70-262:
// io_dr_write_silo_dump) written as a VTK legacy unstructured grid, which
// VisIt (the reference's viewer) and ParaView read.  The Silo library the
// reference writes through (and the HDF5 it sits on) is not available to
// this build; the file holds the same content:
//   - the mesh: node coordinates and each element's four nodes
//     (io_kn_silo_Dmesh);
//   - the materials: each element's material number (ielmat, <= 0 for a
//     mixed cell) and, per material, its volume fraction in every element
//     (1 or 0 for pure elements, frvolume for the components of a mixed
//     cell), the information of the Silo material object
//     (io_kn_silo_Dmaterial, io_kn_set_silo_cp);
//   - the element variables density, energy and pressure (io_kn_silo_DRvar
//     of eldensity, elenergy, elpressure) and the region number (DIvar of
//     ielreg);
//   - the node velocity (ndu, ndv) as one vector.
// Values are printed with 17 significant digits, so they read back bit for
// bit.
#include <cstdio>
#include <stdexcept>

#include "blh_internal.hpp"

namespace blh {

namespace {

void put_scalars(FILE* f, const char* name, const std::vector<double>& v) {
  std::fprintf(f, "SCALARS %s double 1\nLOOKUP_TABLE default\n", name);
  for (double x : v) std::fprintf(f, "%.17g\n", x);
}

void put_ints(FILE* f, const char* name, const std::vector<int>& v) {
  std::fprintf(f, "SCALARS %s int 1\nLOOKUP_TABLE default\n", name);
  for (int x : v) std::fprintf(f, "%d\n", x);
}

std::string field_name(const std::string& s) {
  std::string r;
  for (char c : s) r += (c == ' ' || c == '\t') ? '_' : c;
  return r.empty() ? std::string("unnamed") : r;
}

}  // namespace

void write_vtk(const Problem& p, const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) throw std::runtime_error("cannot open " + path);
  const int nel = p.sizes.nel, nnd = p.sizes.nnd, nmat = p.sizes.nmat;
  const auto& x = p.real.at(BL_NDX);
  const auto& y = p.real.at(BL_NDY);
  const auto& ielnd = p.ints.at(BL_IELND);
  std::fprintf(f, "# vtk DataFile Version 3.0\n");
  std::fprintf(f, "BookLeaf dump nstep=%d time=%.17g\n", p.timestep.nstep, p.timestep.time);
  std::fprintf(f, "ASCII\nDATASET UNSTRUCTURED_GRID\n");
  std::fprintf(f, "POINTS %d double\n", nnd);
  for (int i = 0; i < nnd; i++) std::fprintf(f, "%.17g %.17g 0\n", x[i], y[i]);
  std::fprintf(f, "CELLS %d %d\n", nel, 5 * nel);
  for (int e = 0; e < nel; e++)
    std::fprintf(f, "4 %d %d %d %d\n", ielnd[4 * e] - 1, ielnd[4 * e + 1] - 1,
                 ielnd[4 * e + 2] - 1, ielnd[4 * e + 3] - 1);
  std::fprintf(f, "CELL_TYPES %d\n", nel);
  for (int e = 0; e < nel; e++) std::fprintf(f, "9\n");  // VTK_QUAD
  std::fprintf(f, "CELL_DATA %d\n", nel);
  put_scalars(f, "density", p.real.at(BL_ELDENSITY));
  put_scalars(f, "energy", p.real.at(BL_ELENERGY));
  put_scalars(f, "pressure", p.real.at(BL_ELPRESSURE));
  put_ints(f, "region", p.ints.at(BL_IELREG));
  const auto& ielmat = p.ints.at(BL_IELMAT);
  put_ints(f, "material", ielmat);
  // volume fraction of each material in each element
  std::vector<std::vector<double>> vf(nmat, std::vector<double>(nel, 0.0));
  for (int e = 0; e < nel; e++)
    if (ielmat[e] >= 1 && ielmat[e] <= nmat) vf[ielmat[e] - 1][e] = 1.0;
  if (p.sizes.ncp > 0) {
    const auto& imxel = p.ints.at(BL_IMXEL);
    const auto& imxfcp = p.ints.at(BL_IMXFCP);
    const auto& imxncp = p.ints.at(BL_IMXNCP);
    const auto& icpmat = p.ints.at(BL_ICPMAT);
    const auto& frv = p.real.at(BL_FRVOLUME);
    for (int m = 0; m < p.sizes.nmx; m++) {
      const int e = imxel[m] - 1;
      for (int k = 0; k < imxncp[m]; k++) {
        const int c = imxfcp[m] - 1 + k, mat = icpmat[c];
        if (mat >= 1 && mat <= nmat) vf[mat - 1][e] += frv[c];
      }
    }
  }
  for (int m = 0; m < nmat; m++) {
    const std::string nm = "volume_fraction_" +
                           field_name(m < (int)p.material_names.size() ? p.material_names[m]
                                                                       : std::to_string(m + 1));
    put_scalars(f, nm.c_str(), vf[m]);
  }
  std::fprintf(f, "POINT_DATA %d\nVECTORS velocity double\n", nnd);
  const auto& u = p.real.at(BL_NDU);
  const auto& v = p.real.at(BL_NDV);
  for (int i = 0; i < nnd; i++) std::fprintf(f, "%.17g %.17g 0\n", u[i], v[i]);
  if (std::fclose(f) != 0) throw std::runtime_error("error writing " + path);
}

}  // namespace blh
