// problem.cpp -- the reference's set-up sequence into a Problem, the set-up
// dump, and the host-side reports (short print, Sod check).
#include <cmath>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

#include "blh_internal.hpp"

namespace blh {

Problem problem_from_deck(const std::string& text) {
  const Groups groups = parse_deck(text);
  const Indicators ind = read_indicators(groups);
  Problem p;
  p.config = build_config(groups, ind.nreg, ind.nmat);
  auto mit = groups.find("mesh");
  const MeshData mesh = generate_mesh(mit == groups.end() ? nullptr : &mit->second, p.config.zerocut);
  const InitialState st = apply_initial_conditions(groups, mesh, p.config, ind);
  const int nel = mesh.nel, nnd = mesh.nnd;
  bl_sizes& s = p.sizes;
  s.nel = s.nel1 = s.nel2 = nel;
  s.nnd = s.nnd1 = s.nnd2 = nnd;
  s.nsz = nel > nnd ? nel : nnd;
  s.nmat = ind.nmat;
  s.nreg = ind.nreg;
  s.ncp = st.ncp;
  s.nmx = st.nmx;
  s.mcp = st.ncp;
  s.mmx = st.nmx;
  auto& R = p.real;
  auto& I = p.ints;
  R[BL_ELDENSITY] = st.rho;
  R[BL_ELENERGY] = st.e;
  R[BL_ELPRESSURE] = st.p;
  R[BL_ELCS2] = st.cs2;
  R[BL_ELVOLUME] = st.vol;
  R[BL_A1] = st.a1;
  R[BL_A2] = st.a2;
  R[BL_A3] = st.a3;
  R[BL_B1] = st.b1;
  R[BL_B2] = st.b2;
  R[BL_B3] = st.b3;
  R[BL_CNWT] = st.cnwt;
  R[BL_CNX] = st.cnx;
  R[BL_CNY] = st.cny;
  R[BL_CNVISCX].assign((size_t)nel * 4, 0.0);
  R[BL_CNVISCY].assign((size_t)nel * 4, 0.0);
  R[BL_ELVISC].assign(nel, 0.0);
  R[BL_ELMASS] = st.elmass;
  R[BL_CNMASS] = st.cnmass;
  R[BL_NDX] = mesh.ndx;
  R[BL_NDY] = mesh.ndy;
  R[BL_NDU] = st.u;
  R[BL_NDV] = st.v;
  I[BL_INDTYPE] = mesh.indtype;
  std::vector<int> seq(nel);
  for (int i = 0; i < nel; i++) seq[i] = i + 1;
  I[BL_IELSORT1] = seq;
  I[BL_IELND] = mesh.ielnd;
  I[BL_IELEL] = mesh.ielel;
  I[BL_IELFC] = mesh.ielfc;
  I[BL_IELMAT] = st.ielmat;
  I[BL_IELREG] = st.ielreg;
  if (p.config.ale_zexist) I[BL_IELSORT2] = seq;
  if (p.config.zsp) R[BL_SPMASS] = st.spmass;
  if (st.ncp > 0) {
    const size_t ncp = (size_t)st.ncp;
    R[BL_CPDENSITY] = st.cprho;
    R[BL_CPENERGY] = st.cpe;
    R[BL_CPPRESSURE] = st.cpp;
    R[BL_CPCS2] = st.cpcs2;
    R[BL_CPVOLUME] = st.cpvolume;
    R[BL_FRVOLUME] = st.frvolume;
    R[BL_CPMASS] = st.cpmass;
    R[BL_FRMASS] = st.frmass;
    R[BL_CPVISCX].assign(ncp * 4, 0.0);
    R[BL_CPVISCY].assign(ncp * 4, 0.0);
    R[BL_CPVISC].assign(ncp, 0.0);
    R[BL_CPA1] = st.cpa1;
    R[BL_CPA3] = st.cpa3;
    R[BL_CPB1] = st.cpb1;
    R[BL_CPB3] = st.cpb3;
    I[BL_ICPMAT] = st.icpmat;
    I[BL_IMXEL] = st.imxel;
    I[BL_IMXFCP] = st.imxfcp;
    I[BL_IMXNCP] = st.imxncp;
  }
  // setup_timestep_rationalise
  std::memset(&p.timestep, 0, sizeof p.timestep);
  p.timestep.time = p.config.time_start;
  p.timestep.dt = p.config.dt_initial;
  p.timestep.nstep = 0;
  p.timestep.idtel = -1;
  p.timestep.imdt = -1;
  p.region_names = ind.region_names;
  p.material_names = ind.material_names;
  return p;
}

std::array<void*, BL_NID + 1> Problem::pointer_table() {
  std::array<void*, BL_NID + 1> t{};
  for (auto& kv : real) t[kv.first] = kv.second.data();
  for (auto& kv : ints) t[kv.first] = kv.second.data();
  return t;
}

// Layout: "BLSETUP1", bl_sizes, bl_config, bl_timestep (raw structs), the
// number of fields, then per field: int32 id, int32 kind (0 real, 1 int),
// int64 count, the values.
void write_setup_dump(const Problem& p, const std::string& path) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + path);
  f.write("BLSETUP1", 8);
  f.write(reinterpret_cast<const char*>(&p.sizes), sizeof p.sizes);
  f.write(reinterpret_cast<const char*>(&p.config), sizeof p.config);
  f.write(reinterpret_cast<const char*>(&p.timestep), sizeof p.timestep);
  const int32_t nf = (int32_t)(p.real.size() + p.ints.size());
  f.write(reinterpret_cast<const char*>(&nf), 4);
  for (const auto& kv : p.real) {
    const int32_t id = kv.first, kind = 0;
    const int64_t n = (int64_t)kv.second.size();
    f.write(reinterpret_cast<const char*>(&id), 4);
    f.write(reinterpret_cast<const char*>(&kind), 4);
    f.write(reinterpret_cast<const char*>(&n), 8);
    f.write(reinterpret_cast<const char*>(kv.second.data()), (std::streamsize)(n * 8));
  }
  for (const auto& kv : p.ints) {
    const int32_t id = kv.first, kind = 1;
    const int64_t n = (int64_t)kv.second.size();
    f.write(reinterpret_cast<const char*>(&id), 4);
    f.write(reinterpret_cast<const char*>(&kind), 4);
    f.write(reinterpret_cast<const char*>(&n), 8);
    f.write(reinterpret_cast<const char*>(kv.second.data()), (std::streamsize)(n * 4));
  }
  if (!f) throw std::runtime_error("write failed: " + path);
}

// ------------------------------------------------------------------ reports

std::vector<FlagTotals> shortprint(const Problem& p, bool by_material) {
  const int nflag = by_material ? p.sizes.nmat : p.sizes.nreg;
  std::vector<FlagTotals> t(nflag);
  for (auto& f : t) {  // hydro_kn_init_shortprint
    f.pmx = -DBL_MAX;
    f.pmn = DBL_MAX;
    f.dmx = -DBL_MAX;
    f.dmn = DBL_MAX;
  }
  const auto& flag = p.ints.at(by_material ? BL_IELMAT : BL_IELREG);
  const auto& rho = p.real.at(BL_ELDENSITY);
  const auto& e = p.real.at(BL_ELENERGY);
  const auto& pr = p.real.at(BL_ELPRESSURE);
  const auto& vol = p.real.at(BL_ELVOLUME);
  const auto& m = p.real.at(BL_ELMASS);
  const auto& cnwt = p.real.at(BL_CNWT);
  const auto& u = p.real.at(BL_NDU);
  const auto& v = p.real.at(BL_NDV);
  const auto& nd = p.ints.at(BL_IELND);
  const double dencut = p.config.dencut;
  // hydro_kn_calc_shortprint (hydro_kn_print.F90:52-101); mixed cells
  // (flag <= 0) are skipped here as in the element pass of the reference
  for (int ii = 0; ii < p.sizes.nel; ii++) {
    const int f = flag[ii];
    if (f <= 0 || f > nflag) continue;
    FlagTotals& T = t[f - 1];
    const double c1 = dencut * vol[ii];
    T.vol = T.vol + vol[ii];
    if (m[ii] > c1) {
      double w2 = m[ii];
      T.mass = T.mass + w2;
      double w3 = e[ii];
      w3 = w3 * w2;
      T.ie = T.ie + w3;
      double w4 = pr[ii];
      w3 = w2 * w4;
      T.pressure = T.pressure + w3;
      if (w4 > T.pmx) T.pmx = w4;
      if (w4 < T.pmn) T.pmn = w4;
      w4 = rho[ii];
      if (w4 > T.dmx) T.dmx = w4;
      if (w4 < T.dmn) T.dmn = w4;
      for (int ic = 0; ic < 4; ic++) {
        const int n = nd[(size_t)ii * 4 + ic] - 1;
        w2 = u[n];
        w3 = v[n];
        T.ke = 0.5 * cnwt[(size_t)ii * 4 + ic] * w4 * (w2 * w2 + w3 * w3) + T.ke;
      }
    }
  }
  for (auto& f : t) {  // hydro_kn_average_shortprint (hydro_kn_print.F90:219-240)
    f.density = f.vol > 0.0 ? f.mass / f.vol : 0.0;
    if (f.mass > dencut * f.vol) f.pressure = f.pressure / f.mass;
  }
  return t;
}

std::string format_shortprint(const Problem& p, int nstep, double time) {
  return format_shortprint(p, nstep, time, shortprint(p, false), shortprint(p, true));
}

std::string format_shortprint(const Problem& p, int nstep, double time,
                              const std::vector<FlagTotals>& reg,
                              const std::vector<FlagTotals>& matl) {
  std::ostringstream o;
  char buf[512];
  std::snprintf(buf, sizeof buf, "\n  Step no. %7d Time = %14.7f\n", nstep, time);
  o << buf;
  double tv = 0, tm = 0, tie = 0, tke = 0, tp = 0;
  for (int pass = 0; pass < 2; pass++) {
    const bool mat = pass == 1;
    const auto& t = mat ? matl : reg;
    o << "\n" << (mat ? " Material" : " Region") << " summary\n\n";
    std::snprintf(buf, sizeof buf, "  %-10s %11s %11s %11s %11s %11s %11s %11s %11s %11s %11s\n",
                  mat ? "material" : "region", "vol", "mass", "tot ie", "tot ke", "press",
                  "min press", "max press", "dens", "min dens", "max dens");
    o << buf;
    const auto& names = mat ? p.material_names : p.region_names;
    for (size_t i = 0; i < t.size(); i++) {
      const auto& f = t[i];
      std::snprintf(buf, sizeof buf,
                    "  %-10.10s %11.4e %11.4e %11.4e %11.4e %11.4e %11.4e %11.4e %11.4e %11.4e %11.4e\n",
                    i < names.size() ? names[i].c_str() : "", f.vol, f.mass, f.ie, f.ke,
                    f.pressure, f.pmn, f.pmx, f.density, f.dmn, f.dmx);
      o << buf;
      if (!mat) {
        tv += f.vol;
        tm += f.mass;
        tie += f.ie;
        tke += f.ke;
        tp += f.pressure * f.mass;
      }
    }
  }
  std::snprintf(buf, sizeof buf,
                "\n Total      %11.4e %11.4e %11.4e %11.4e %11.4e\n"
                "\n           total energy\n internal  %11.4e\n kinetic   %11.4e\n total     %11.4e\n",
                tv, tm, tie, tke, tm > 0 ? tp / tm : 0.0, tie, tke, tie + tke);
  o << buf;
  return o.str();
}

namespace {

// sod (check_kn_tests.f90:64-111): exact density and energy of the Sod
// problem at x (relative to the interface) and time t, gamma = 1.4
void sod_exact(double xx, double time, double& rho, double& e) {
  rho = -DBL_MAX;
  e = -DBL_MAX;
  const double coeff = std::sqrt(1.4);
  if (xx <= -coeff * time) {
    rho = 1.0;
    e = 2.5;
  } else if (xx <= -0.07027281256118326961 * time) {
    const double ss = xx / time;
    const double velocity = (5.0 / 6.0) * (ss + coeff);
    const double tt = ((velocity - ss) * (velocity - ss)) / 1.4;
    rho = std::pow(tt, 2.5);
    e = rho * tt / (0.4 * rho);
  } else if (xx <= 0.92745262004894994908 * time) {
    rho = 0.42631942817849519385;
    e = 1.77760006942335264781;
  } else if (time <= 28.53627624872492075028) {
    if (xx <= 1.75215573203017816370 * time) {
      rho = 0.26557371170530706471;
      e = 2.85354088799095973738;
    } else {
      rho = 0.125;
      e = 2.0;
    }
  } else if (time < 40.68191725689148697880) {
    if (xx <= (50.0 - (time - 28.53627624872492075028) * 1.01019363599101820444)) {
      rho = 0.26557371170530706471;
      e = 2.85354088799095973738;
    } else {
      rho = 0.50939531774381657731;
      e = 3.82996297061558546292;
    }
  }
}

}  // namespace

void check_sod(const Problem& p, double time, double& l1_density, double& l1_energy) {
  const auto& vol = p.real.at(BL_ELVOLUME);
  const auto& rho = p.real.at(BL_ELDENSITY);
  const auto& e = p.real.at(BL_ELENERGY);
  const auto& x = p.real.at(BL_NDX);
  const auto& y = p.real.at(BL_NDY);
  const auto& nd = p.ints.at(BL_IELND);
  double basis = 0.0, l1d = 0.0, l1e = 0.0;
  for (int ii = 0; ii < p.sizes.nel; ii++) {
    double xx[4], yy[4];
    for (int c = 0; c < 4; c++) {
      xx[c] = x[nd[(size_t)ii * 4 + c] - 1];
      yy[c] = y[nd[(size_t)ii * 4 + c] - 1];
    }
    // geometry_kn_getcentroid
    double cx = 0, cy = 0, rvol = 0;
    for (int i1 = 0; i1 < 4; i1++) {
      const int i2 = (i1 + 1) % 4;
      const double rr = xx[i1] * yy[i2] - xx[i2] * yy[i1];
      rvol = rvol + rr;
      cx = cx + rr * (xx[i1] + xx[i2]);
      cy = cy + rr * (yy[i1] + yy[i2]);
    }
    rvol = 0.5 * rvol;
    cx = rvol > 0.0 ? cx / (6.0 * rvol) : 0.0;
    double sr, se;
    sod_exact(cx - 50.0, time, sr, se);
    basis = basis + vol[ii];
    l1d = std::fabs(rho[ii] - sr) * vol[ii] + l1d;
    l1e = std::fabs(e[ii] - se) * vol[ii] + l1e;
  }
  l1_density = l1d / basis;
  l1_energy = l1e / basis;
}

}  // namespace blh
