// blh_internal.hpp -- set-up pieces shared between the host sources.
#pragma once

#include "blh.hpp"

namespace blh {

// A single-partition mesh in the reference's numbering (1-based ids);
// ielnd/ielel/ielfc are (NCORN,nel) blocks.
struct MeshData {
  int nel = 0, nnd = 0;
  std::vector<double> ndx, ndy;
  std::vector<int> indtype, ielnd, ielel, ielfc, ielreg, ielmat;
};

MeshData generate_mesh(const Namelist* mesh_nl, double zerocut);
void connectivity(const std::vector<int>& ielnd, int nel, std::vector<int>& ielel,
                  std::vector<int>& ielfc);
void nodetype(const std::vector<int>& ielnd, int nel, std::vector<int>& indtype);

// An indicator of setup_indicator_types: (type, value, number).
struct Indicator {
  std::string type;
  int value;
  int number;
};

struct Indicators {
  int nreg = 0, nmat = 0;
  std::vector<Indicator> regions, materials;
  bool rmesh = false, mmesh = false;
  std::vector<std::string> region_names, material_names;
};

Indicators read_indicators(const Groups& groups);

// The initial state of setup_IC + init (element, corner, node and
// component fields).
struct InitialState {
  int nmx = 0, ncp = 0;
  std::vector<int> ielreg, ielmat, imxel, imxfcp, imxncp, icpmat;
  std::vector<double> cnx, cny, a1, a2, a3, b1, b2, b3, cnwt, vol, rho, e, u, v;
  std::vector<double> elmass, cnmass, p, cs2, spmass;
  std::vector<double> frvolume, cpvolume, cprho, cpe, cpmass, frmass, cpp, cpcs2;
  std::vector<double> cpa1, cpa3, cpb1, cpb3;
};

InitialState apply_initial_conditions(const Groups& groups, const MeshData& mesh,
                                      const bl_config& cfg, const Indicators& ind);

}  // namespace blh
