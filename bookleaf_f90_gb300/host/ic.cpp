// ic.cpp -- initial conditions and initial state, in the order inf_init runs
// them (inf_init.F90:53-103):
//
//   setup_indicator_types / setup_shapes_type / setup_IC_type
//                              setup_IC.f90:813-1419 (INDICATORS, SHAPES,
//                                                     INITIAL_CONDITIONS)
//   setup_regions / setup_materials / setup_flag*
//                              setup_IC.f90:268-593, region_shape and
//                              material_shape 1553-1636, intersect and
//                              subdivide 1660-1730
//   mix list + flatten         mix_dr_list.f90:46-205 (components of a mixed
//                              cell contiguous, mixed cells in cell order)
//   setup_state                setup_IC.f90:321-431
//   init_dr_state              init_dr_utils.f90:95-132 (masses, EoS)
//   hydro_dr_init              hydro_dr_init.f90:38-59 (spmass)
#include <algorithm>
#include <cmath>
#include <map>
#include <set>

#include "blh_internal.hpp"

namespace blh {

namespace {

constexpr int LN = 100;
constexpr int MAXIT = 10;

struct Shape {
  std::string type;  // RECTANGLE or CIRCLE
  double p[5];
};

struct Thermo {
  std::string itype, scale;
  int param;
  double density, energy;
};

struct Kinematic {
  std::string itype, geom;
  int param;
  double dat[3];
};

std::vector<Shape> read_shapes(const Groups& groups) {
  static const Namelist empty;
  auto it = groups.find("shapes");
  const Namelist& sh = it == groups.end() ? empty : it->second;
  const auto stype = sh.get_array("shape_type", {LN}, Value::str("UNKNOWN"));
  const auto sparam = sh.get_array("shape_param", {LN, 5}, Value::real(0.0));
  std::vector<Shape> forms;
  for (int i = 0; i < LN; i++) {
    const std::string t = stype[i].as_str();
    if (t == "UNKNOWN") continue;
    Shape s;
    s.type = t;
    for (int q = 0; q < 5; q++) s.p[q] = sparam[(size_t)i * 5 + q].as_real();
    if (t == "CIRCLE") s.p[3] = 0.0;
    else if (t != "RECTANGLE") throw DeckError("ERROR: unrecognised shape type");
    forms.push_back(s);
  }
  return forms;
}

void read_ic(const Groups& groups, std::vector<Thermo>& thermo, std::vector<Kinematic>& kin) {
  static const Namelist empty;
  auto it = groups.find("initial_conditions");
  const Namelist& ic = it == groups.end() ? empty : it->second;
  const auto ttype = ic.get_array("thermodynamic_type", {LN}, Value::str("UNKNOWN"));
  const auto tval = ic.get_array("thermodynamic_value", {LN}, Value::integer(-1));
  const auto tscale = ic.get_array("thermodynamic_energy_scale", {LN}, Value::str("UNKNOWN"));
  const auto dens = ic.get_array("density", {LN}, Value::real(-1.0));
  const auto ener = ic.get_array("energy", {LN}, Value::real(-1.0));
  for (int i = 0; i < LN; i++) {
    const std::string t = ttype[i].as_str();
    if (t == "UNKNOWN") continue;
    if (t != "REGION" && t != "MATERIAL") throw DeckError("ERROR: unrecognised thermodynamic type");
    if (dens[i].as_real() <= 0.0) throw DeckError("ERROR: density <= 0");
    if (ener[i].as_real() < 0.0) throw DeckError("ERROR: energy < 0");
    thermo.push_back({t, tscale[i].as_str(), (int)tval[i].as_int(), dens[i].as_real(),
                      ener[i].as_real()});
  }
  if (thermo.empty()) throw DeckError("ERROR: No initial conditions defined");
  const auto ktype = ic.get_array("kinematic_type", {LN}, Value::str("UNKNOWN"));
  const auto kgeom = ic.get_array("kinematic_geometry", {LN}, Value::str("UNKNOWN"));
  const auto kval = ic.get_array("kinematic_value", {LN}, Value::integer(-1));
  const auto kpar = ic.get_array("kinematic_param", {3, LN}, Value::real(0.0));
  for (int i = 0; i < LN; i++) {
    const std::string t = ktype[i].as_str();
    if (t == "UNKNOWN") continue;
    if (t != "BACKGROUND" && t != "REGION") throw DeckError("ERROR: unrecognised kinematic type");
    Kinematic k;
    k.itype = t;
    k.geom = kgeom[i].as_str();
    k.param = (int)kval[i].as_int();
    for (int j = 0; j < 3; j++) k.dat[j] = kpar[(size_t)j * LN + i].as_real();
    if (k.geom == "PLANAR") k.dat[2] = 0.0;
    else if (k.geom != "RADIAL") throw DeckError("ERROR: unrecognised kinematic geometry");
    kin.push_back(k);
  }
}

// geometry_kn_getcentroid (geometry_kn_centroid.f90:29-55) of n vertices
void centroid(int n, const double* xx, const double* yy, double& cx, double& cy) {
  cx = 0.0;
  cy = 0.0;
  double rvol = 0.0;
  for (int i1 = 0; i1 < n; i1++) {
    const int i2 = (i1 + 1) % n;
    const double rr = xx[i1] * yy[i2] - xx[i2] * yy[i1];
    rvol = rvol + rr;
    cx = cx + rr * (xx[i1] + xx[i2]);
    cy = cy + rr * (yy[i1] + yy[i2]);
  }
  rvol = 0.5 * rvol;
  if (rvol > 0.0) {
    cx = cx / (6.0 * rvol);
    cy = cy / (6.0 * rvol);
  } else {
    cx = 0.0;
    cy = 0.0;
  }
}

bool inside(const Shape& s, double px, double py) {
  if (s.type == "RECTANGLE") return px > s.p[0] && py > s.p[1] && px < s.p[2] && py < s.p[3];
  const double dx = px - s.p[0], dy = py - s.p[1];
  return std::sqrt(dx * dx + dy * dy) <= s.p[2];
}

double intersect(const Shape& s, const double* xx, const double* yy) {
  int in = 0;
  for (int i = 0; i < 4; i++) in += inside(s, xx[i], yy[i]) ? 1 : 0;
  return in == 4 ? 1.0 : (in > 0 ? 0.5 : 0.0);
}

// subdivide (setup_IC.f90:1682-1730)
double subdivide(int nit, const Shape& s, const double* xx, const double* yy) {
  const int nit_local = nit + 1;
  double cx, cy;
  centroid(4, xx, yy, cx, cy);
  if (nit_local > MAXIT) return inside(s, cx, cy) ? 1.0 : 0.0;
  double vf = 0.0;
  for (int ii = 0; ii < 4; ii++) {
    const int jj = (ii + 1) % 4, kk = (ii + 3) % 4;
    const double xl[4] = {xx[ii], xx[jj], cx, xx[kk]};
    const double yl[4] = {yy[ii], yy[jj], cy, yy[kk]};
    double v = intersect(s, xl, yl);
    if (v > 0.25 && v < 0.75) v = subdivide(nit_local, s, xl, yl);
    vf = vf + v;
  }
  return 0.25 * vf;
}

// setup_flag (setup_IC.f90:433-486) for regions (mix null) or materials
// (mix collects the mixed cells, material_shape)
void flag(const std::vector<Indicator>& inds, std::vector<int>& iflag, const std::vector<int>& itest,
          const std::vector<double>& cnx, const std::vector<double>& cny,
          const std::vector<Shape>& forms, std::map<int, std::vector<std::pair<int, double>>>* mix) {
  const int n = (int)iflag.size();
  for (const auto& ind : inds) {
    if (ind.type == "MESH") break;
    if (ind.type == "BACKGROUND") {
      std::fill(iflag.begin(), iflag.end(), ind.number);
    } else if (ind.type == "CELL") {
      if (ind.value < 1 || ind.value > n) throw DeckError("ERROR: incorrect cell index in setup_flag_cell");
      iflag[ind.value - 1] = ind.number;
    } else if (ind.type == "REGION" || ind.type == "MATERIAL") {
      for (int i = 0; i < n; i++)
        if (itest[i] == ind.value) iflag[i] = ind.number;
    } else if (ind.type == "SHAPE") {
      if (ind.value < 1 || ind.value > (int)forms.size()) throw DeckError("ERROR: failed to find shape");
      const Shape& s = forms[ind.value - 1];
      if (!mix) {
        for (int i = 0; i < n; i++) {
          double px, py;
          centroid(4, &cnx[(size_t)i * 4], &cny[(size_t)i * 4], px, py);
          if (inside(s, px, py)) iflag[i] = ind.number;
        }
      } else {
        for (int i = 0; i < n; i++) {
          double vf = intersect(s, &cnx[(size_t)i * 4], &cny[(size_t)i * 4]);
          if (vf > 0.75) {
            iflag[i] = ind.number;
          } else if (vf > 0.25) {
            vf = s.p[4] > 0.0 ? s.p[4] : subdivide(0, s, &cnx[(size_t)i * 4], &cny[(size_t)i * 4]);
            const int jj = iflag[i];
            if (jj > 0) {
              (*mix)[i + 1] = {{jj, 1.0 - vf}};
              iflag[i] = -1;
            }
            (*mix)[i + 1].push_back({ind.number, vf});
          }
        }
      }
    } else {
      throw DeckError("ERROR: unrecognised indicator type");
    }
  }
}

// setup_thermodynamic (setup_IC.f90:595-629)
void thermo_set(const Thermo& t, const std::vector<int>& iflag, const std::vector<double>& vol,
                std::vector<double>& rho, std::vector<double>& e) {
  for (size_t i = 0; i < iflag.size(); i++) {
    if (iflag[i] != t.param) continue;
    rho[i] = t.density;
    e[i] = t.energy;
    if (t.scale == "VOLUME") e[i] = e[i] / vol[i];
    else if (t.scale == "MASS") e[i] = e[i] / (rho[i] * vol[i]);
  }
}

// eos_kn_getpressure / eos_kn_getcs2 (eos_kn_forms.f90:28-106)
void eos(const bl_config& cfg, const std::vector<int>& imat_in, const std::vector<double>& rho,
         const std::vector<double>& e, std::vector<double>& p, std::vector<double>& c2) {
  const size_t n = rho.size();
  p.assign(n, 0.0);
  c2.assign(n, 0.0);
  for (size_t i = 0; i < n; i++) {
    const int m = std::max(imat_in[i], 0);
    const int t = cfg.eos_type[m];
    const double* P = cfg.eos_param[m];
    const double r = rho[i], en = e[i];
    double pp, cc;
    if (t == 0) {
      pp = P[0];
      cc = cfg.ccut;
    } else if (t == 1) {
      pp = en * r * (P[0] - 1.0);
      cc = P[0] * (P[0] - 1.0) * en;
    } else if (t == 2) {
      const double t1 = r / P[2];
      pp = P[0] * (std::pow(t1, P[1]) - 1.0);
      pp = P[3] > pp ? P[3] : pp;
      cc = (P[0] * P[1]) / P[2] * std::pow(t1, P[1] - 1.0);
    } else if (t == 3) {
      const double t1 = P[3] * P[5] / r;
      const double t2 = P[4] * P[5] / r;
      pp = P[0] * r * en + (1.0 - P[0] / t1) * P[1] * std::exp(-t1) +
           (1.0 - P[0] / t2) * P[2] * std::exp(-t2);
      if (std::fabs(pp) < cfg.pcut) pp = 0.0;
      const double q1 = P[5] / r;
      double s3 = P[3] * q1;
      const double t4 = (P[0] / P[3] + P[0] * q1 - s3 * q1) * P[1] * std::exp(-s3);
      s3 = P[4] * q1;
      const double t5 = (P[0] / P[4] + P[0] * q1 - s3 * q1) * P[2] * std::exp(-s3);
      cc = P[0] * pp / r + P[0] * en - t4 - t5;
    } else {
      pp = -1.0;
      cc = cfg.ccut;
    }
    if (std::fabs(pp) < cfg.pcut) pp = 0.0;
    if (cfg.ccut > cc) cc = cfg.ccut;
    p[i] = pp;
    c2[i] = cc;
  }
}

}  // namespace

Indicators read_indicators(const Groups& groups) {
  static const Namelist empty;
  auto it = groups.find("indicators");
  const Namelist& nl = it == groups.end() ? empty : it->second;
  const auto rt = nl.get_array("region_type", {LN}, Value::str("UNKNOWN"));
  const auto rv = nl.get_array("region_value", {LN}, Value::integer(-1));
  const auto mt = nl.get_array("material_type", {LN}, Value::str("UNKNOWN"));
  const auto mv = nl.get_array("material_value", {LN}, Value::integer(-1));
  const auto rn = nl.get_array("region_name", {LN}, Value::str(""));
  const auto mn = nl.get_array("material_name", {LN}, Value::str(""));
  Indicators ind;
  std::vector<std::string> rtype, mtype;
  std::vector<int> rval, mval;
  for (int i = 0; i < LN; i++) {
    if (rt[i].as_str() != "UNKNOWN") ind.nreg++;
    if (mt[i].as_str() != "UNKNOWN") ind.nmat++;
  }
  if (ind.nreg < 1) throw DeckError("ERROR: No regions defined");
  if (ind.nmat < 1) throw DeckError("ERROR: No materials defined");
  for (int i = 0; i < ind.nreg; i++) {
    rtype.push_back(rt[i].as_str());
    rval.push_back((int)rv[i].as_int());
    ind.region_names.push_back(rn[i].kind == Value::STR ? rn[i].s : "");
  }
  for (int i = 0; i < ind.nmat; i++) {
    mtype.push_back(mt[i].as_str());
    mval.push_back((int)mv[i].as_int());
    ind.material_names.push_back(mn[i].kind == Value::STR ? mn[i].s : "");
  }
  auto all_mesh = [](const std::vector<std::string>& v) {
    return std::all_of(v.begin(), v.end(), [](const std::string& t) { return t == "MESH"; });
  };
  auto any_mesh = [](const std::vector<std::string>& v) {
    return std::any_of(v.begin(), v.end(), [](const std::string& t) { return t == "MESH"; });
  };
  if (any_mesh(rtype) && !all_mesh(rtype))
    throw DeckError("ERROR: Cannot mix region type MESH with other region types");
  if (any_mesh(mtype) && !all_mesh(mtype))
    throw DeckError("ERROR: Cannot mix material type MESH with other material types");
  auto order = [](const std::vector<std::string>& types, const std::vector<int>& vals,
                  const std::string& third, const char* what) {
    std::vector<Indicator> out;
    for (size_t i = 0; i < types.size(); i++)
      if (types[i] == "BACKGROUND") out.push_back({"BACKGROUND", vals[i], (int)i + 1});
    for (size_t i = 0; i < types.size(); i++)
      if (types[i] == "CELL" || types[i] == "MESH" || types[i] == third)
        out.push_back({types[i], vals[i], (int)i + 1});
    for (size_t i = 0; i < types.size(); i++)
      if (types[i] == "SHAPE") out.push_back({"SHAPE", vals[i], (int)i + 1});
    for (const auto& t : types)
      if (t != "BACKGROUND" && t != "CELL" && t != "MESH" && t != third && t != "SHAPE")
        throw DeckError(std::string("ERROR: unrecognised value of ") + what + "_type");
    return out;
  };
  ind.regions = order(rtype, rval, "MATERIAL", "region");
  ind.materials = order(mtype, mval, "REGION", "material");
  ind.rmesh = all_mesh(rtype);
  ind.mmesh = all_mesh(mtype);
  return ind;
}

InitialState apply_initial_conditions(const Groups& groups, const MeshData& mesh,
                                      const bl_config& cfg, const Indicators& ind) {
  const std::vector<Shape> forms = read_shapes(groups);
  std::vector<Thermo> thermo;
  std::vector<Kinematic> kin;
  read_ic(groups, thermo, kin);
  const int nel = mesh.nel, nnd = mesh.nnd;
  InitialState st;
  st.cnx.resize((size_t)nel * 4);
  st.cny.resize((size_t)nel * 4);
  for (size_t c = 0; c < (size_t)nel * 4; c++) {
    st.cnx[c] = mesh.ndx[mesh.ielnd[c] - 1];
    st.cny[c] = mesh.ndy[mesh.ielnd[c] - 1];
  }
  // setup_regions (setup_IC.f90:268-290)
  st.ielreg = ind.rmesh ? mesh.ielreg : std::vector<int>(nel, 0);
  flag(ind.regions, st.ielreg, mesh.ielmat, st.cnx, st.cny, forms, nullptr);
  for (int v : st.ielreg)
    if (v == 0) throw DeckError("ERROR: region not fully populated");
  // setup_materials (setup_IC.f90:292-319)
  st.ielmat = ind.mmesh ? mesh.ielmat : std::vector<int>(nel, 0);
  std::map<int, std::vector<std::pair<int, double>>> mix;  // 1-based cell -> (material, fraction)
  flag(ind.materials, st.ielmat, st.ielreg, st.cnx, st.cny, forms, &mix);
  for (int v : st.ielmat)
    if (v == 0) throw DeckError("ERROR: material not fully populated");
  // flatten: mixed cells in cell order, their components contiguous
  st.nmx = (int)mix.size();
  std::vector<int> cp_el;  // 1-based element of each component
  int fcp = 1;
  for (const auto& kv : mix) {
    st.imxel.push_back(kv.first);
    st.imxncp.push_back((int)kv.second.size());
    st.imxfcp.push_back(fcp);
    fcp += (int)kv.second.size();
    for (const auto& mf : kv.second) {
      st.icpmat.push_back(mf.first);
      st.frvolume.push_back(mf.second);
      cp_el.push_back(kv.first);
    }
  }
  st.ncp = (int)st.icpmat.size();
  for (int imx = 0; imx < st.nmx; imx++) st.ielmat[st.imxel[imx] - 1] = -(imx + 1);
  // setup_state: geometry (geometry_kn_getiso/getvolume,
  // geometry_kn_volume.f90:30-79)
  st.a1.resize(nel); st.a2.resize(nel); st.a3.resize(nel);
  st.b1.resize(nel); st.b2.resize(nel); st.b3.resize(nel);
  st.cnwt.resize((size_t)nel * 4);
  st.vol.resize(nel);
  const double o9 = 1.0 / 9.0;
  for (int i = 0; i < nel; i++) {
    const double* x = &st.cnx[(size_t)i * 4];
    const double* y = &st.cny[(size_t)i * 4];
    const double a1 = 0.25 * ((((-x[0]) + x[1]) + x[2]) - x[3]);
    const double a2 = 0.25 * ((((x[0] - x[1]) + x[2]) - x[3]));
    const double a3 = 0.25 * ((((-x[0]) - x[1]) + x[2]) + x[3]);
    const double b1 = 0.25 * ((((-y[0]) + y[1]) + y[2]) - y[3]);
    const double b2 = 0.25 * ((((y[0] - y[1]) + y[2]) - y[3]));
    const double b3 = 0.25 * ((((-y[0]) - y[1]) + y[2]) + y[3]);
    st.a1[i] = a1; st.a2[i] = a2; st.a3[i] = a3;
    st.b1[i] = b1; st.b2[i] = b2; st.b3[i] = b3;
    double* w = &st.cnwt[(size_t)i * 4];
    w[0] = o9 * ((3.0 * b3 - b2) * (3.0 * a1 - a2) - (3.0 * a3 - a2) * (3.0 * b1 - b2));
    w[1] = o9 * ((3.0 * b3 + b2) * (3.0 * a1 - a2) - (3.0 * a3 + a2) * (3.0 * b1 - b2));
    w[2] = o9 * ((3.0 * b3 + b2) * (3.0 * a1 + a2) - (3.0 * a3 + a2) * (3.0 * b1 + b2));
    w[3] = o9 * ((3.0 * b3 - b2) * (3.0 * a1 + a2) - (3.0 * a3 - a2) * (3.0 * b1 + b2));
    st.vol[i] = 4.0 * (a1 * b3 - a3 * b1);
    if (st.vol[i] < 0.0) throw DeckError("ERROR: negative volume in geometry_dr_getgeometry");
  }
  st.cpvolume.resize(st.ncp);
  for (int c = 0; c < st.ncp; c++) {
    const int i = cp_el[c] - 1;
    st.cpvolume[c] = (4.0 * (st.a1[i] * st.b3[i] - st.a3[i] * st.b1[i])) * st.frvolume[c];
  }
  st.rho.assign(nel, 0.0);
  st.e.assign(nel, 0.0);
  st.cprho.assign(st.ncp, 0.0);
  st.cpe.assign(st.ncp, 0.0);
  bool any_region = false;
  for (const auto& t : thermo) {
    if (t.itype == "REGION") {
      any_region = true;
      thermo_set(t, st.ielreg, st.vol, st.rho, st.e);
    } else {
      thermo_set(t, st.ielmat, st.vol, st.rho, st.e);
      if (st.ncp) thermo_set(t, st.icpmat, st.cpvolume, st.cprho, st.cpe);
    }
  }
  if (st.ncp && any_region) {
    // setup_thermodynamic_rationalise (setup_IC.f90:740-787)
    std::set<int> matset;
    for (const auto& t : thermo)
      if (t.itype == "MATERIAL") matset.insert(t.param);
    std::map<int, std::string> mtypes;
    for (const auto& m : ind.materials) mtypes[m.number] = m.type;
    for (int c = 0; c < st.ncp; c++) {
      const int m = st.icpmat[c];
      if (matset.count(m)) continue;
      auto mt = mtypes.find(m);
      if (mt != mtypes.end() && (mt->second == "REGION" || mt->second == "BACKGROUND")) {
        st.cprho[c] = st.rho[cp_el[c] - 1];
        st.cpe[c] = st.e[cp_el[c] - 1];
      } else {
        throw DeckError(
            "ERROR: failed to rationalise thermodynamic IC due to incorrect material type");
      }
    }
  }
  // kinematics (setup_IC.f90:372-380, 631-811)
  st.u.assign(nnd, 0.0);
  st.v.assign(nnd, 0.0);
  bool any_kreg = false;
  for (const auto& k : kin) any_kreg = any_kreg || k.itype == "REGION";
  std::vector<double> wt(any_kreg ? nnd : 0, 0.0);
  for (const auto& k : kin) {
    const double* d = k.dat;
    if (k.itype == "BACKGROUND") {
      for (int n = 0; n < nnd; n++) {
        if (k.geom == "RADIAL") {
          const double dx = mesh.ndx[n] - d[1], dy = mesh.ndy[n] - d[2];
          const double rv = 1.0 / std::sqrt(dx * dx + dy * dy);
          st.u[n] = d[0] * mesh.ndx[n] * rv;
          st.v[n] = d[0] * mesh.ndy[n] * rv;
        } else {
          st.u[n] = d[0];
          st.v[n] = d[1];
        }
      }
    } else {
      for (int iel = 0; iel < nel; iel++) {
        if (st.ielreg[iel] != k.param) continue;
        double px = 0, py = 0, rv = 0;
        if (k.geom == "RADIAL") {
          centroid(4, &st.cnx[(size_t)iel * 4], &st.cny[(size_t)iel * 4], px, py);
          const double dx = px - d[1], dy = py - d[2];
          rv = 1.0 / std::sqrt(dx * dx + dy * dy);
        }
        for (int ic = 0; ic < 4; ic++) {
          const int n = mesh.ielnd[(size_t)iel * 4 + ic] - 1;
          const double w = st.cnwt[(size_t)iel * 4 + ic];
          if (k.geom == "RADIAL") {
            st.u[n] = st.u[n] + w * px * rv * d[0];
            st.v[n] = st.v[n] + w * py * rv * d[1];
          } else {
            st.u[n] = st.u[n] + w * d[0];
            st.v[n] = st.v[n] + w * d[1];
          }
          wt[n] = wt[n] + w;
        }
      }
    }
  }
  if (any_kreg) {
    for (int n = 0; n < nnd; n++) {
      if (std::fabs(wt[n]) < cfg.zerocut) {
        st.u[n] = 0.0;
        st.v[n] = 0.0;
      } else {
        const double rv = 1.0 / wt[n];
        st.u[n] = st.u[n] * rv;
        st.v[n] = st.v[n] * rv;
      }
    }
  }
  // utils_dr_bc with accut (utils_kn_bc.f90:28-58)
  for (int n = 0; n < nnd; n++) {
    const int t = mesh.indtype[n];
    if (t == -1 || t == -3) st.u[n] = 0.0;
    if (t == -2 || t == -3) st.v[n] = 0.0;
    const double w2 = st.u[n] * st.u[n] + st.v[n] * st.v[n];
    if (w2 < cfg.accut * cfg.accut) {
      st.u[n] = 0.0;
      st.v[n] = 0.0;
    }
  }
  for (int i = 0; i < nel; i++) {
    if (st.rho[i] <= 0.0) throw DeckError("ERROR: eldensity not positive");
    if (st.e[i] < 0.0) throw DeckError("ERROR: elenergy negative");
  }
  // init_dr_state: masses (init_kn.f90:32-63) and EoS
  st.elmass.resize(nel);
  st.cnmass.resize((size_t)nel * 4);
  for (int i = 0; i < nel; i++) {
    st.elmass[i] = st.rho[i] * st.vol[i];
    for (int c = 0; c < 4; c++) st.cnmass[(size_t)i * 4 + c] = st.rho[i] * st.cnwt[(size_t)i * 4 + c];
  }
  st.cpmass.resize(st.ncp);
  st.frmass.resize(st.ncp);
  for (int c = 0; c < st.ncp; c++) {
    st.cpmass[c] = st.cprho[c] * st.cpvolume[c];
    st.frmass[c] = st.cpmass[c] / st.elmass[cp_el[c] - 1];
  }
  eos(cfg, st.ielmat, st.rho, st.e, st.p, st.cs2);
  if (st.ncp) eos(cfg, st.icpmat, st.cprho, st.cpe, st.cpp, st.cpcs2);
  // hydro_dr_init: spmass (hydro_kn_init.f90:46-77)
  if (cfg.zsp) {
    st.spmass.resize((size_t)nel * 4);
    for (int i = 0; i < nel; i++) {
      const double* cx = &st.cnx[(size_t)i * 4];
      const double* cy = &st.cny[(size_t)i * 4];
      const double x3 = 0.25 * (((cx[0] + cx[1]) + cx[2]) + cx[3]);
      const double y3 = 0.25 * (((cy[0] + cy[1]) + cy[2]) + cy[3]);
      for (int j1 = 0; j1 < 4; j1++) {
        const double x1 = cx[j1], y1 = cy[j1];
        int j2 = (j1 + 1) % 4;
        const double x2 = 0.5 * (x1 + cx[j2]), y2 = 0.5 * (y1 + cy[j2]);
        j2 = (j1 + 3) % 4;
        const double x4 = 0.5 * (x1 + cx[j2]), y4 = 0.5 * (y1 + cy[j2]);
        const double w1 = 0.25 * ((((-x1) + x2) + x3) - x4);
        const double w2 = 0.25 * ((((-x1) - x2) + x3) + x4);
        const double w3 = 0.25 * ((((-y1) + y2) + y3) - y4);
        const double w4 = 0.25 * ((((-y1) - y2) + y3) + y4);
        st.spmass[(size_t)i * 4 + j1] = 4.0 * st.rho[i] * (w1 * w4 - w2 * w3);
      }
    }
  }
  st.cpa1.resize(st.ncp); st.cpa3.resize(st.ncp);
  st.cpb1.resize(st.ncp); st.cpb3.resize(st.ncp);
  for (int c = 0; c < st.ncp; c++) {
    const int i = cp_el[c] - 1;
    st.cpa1[c] = st.a1[i];
    st.cpa3[c] = st.a3[i];
    st.cpb1[c] = st.b1[i];
    st.cpb3[c] = st.b3[i];
  }
  return st;
}

}  // namespace blh
