// mesh.cpp -- structured-region mesh generator, numbering, connectivity and
// node types (host side, before the hot path):
//
//   setup_mesh_read_input   setup_mesh.F90:106-346   (MESH namelist)
//   setup_mesh_region       setup_mesh.F90:593-1089  (LIN1/LIN2 weights, side
//                                                     lines, interior guess and
//                                                     relaxation, corner BCs)
//   setup_mesh_line         setup_mesh.F90:1750-1855
//   setup_mesh_arc          setup_mesh.F90:1857-2062
//   setup_mesh_transfer     setup_mesh.F90:1091-1250 (node/element numbering)
//   utils_kn_getconn/getsconn/corrconn   utils_kn_connectivity.f90:30-170
//   init_kn_nodetype        init_kn.f90:78-106
//
// One mesh region of type LIN1 or LIN2 whose four sides are single LINE,
// LINK, ARC_A or ARC_C segments: every deck of the reference.  Node l runs along region_dim(:,2), k along region_dim(:,1), as the
// reference stores them, so node and element numbers match the reference's.
#include <algorithm>
#include <cmath>
#include <set>

#include "blh_internal.hpp"

namespace blh {

namespace {

constexpr int LI = 100;

int bc_code(const std::string& b) {
  if (b == "SLIPX") return 1;
  if (b == "SLIPY") return 2;
  if (b == "WALL") return 3;
  if (b == "TRANS") return 6;
  if (b == "OPEN") return 7;
  if (b == "FREE") return 8;
  throw DeckError("ERROR: unrecognised segment boundary condition");
}

struct Grid {  // (no_l, no_k) arrays, index (l-1)*no_k + (k-1)
  int no_l, no_k;
  std::vector<double> rr, ss;
  std::vector<int> bc;
  double& r(int l, int k) { return rr[(size_t)l * no_k + k]; }  // 0-based
  double& s(int l, int k) { return ss[(size_t)l * no_k + k]; }
  int& b(int l, int k) { return bc[(size_t)l * no_k + k]; }
};

// setup_mesh_line (setup_mesh.F90:1750-1855) for one side
void side_line(Grid& g, const double* point, int segbc, int ind, double zerocut, double tol,
               double om, int rtyp) {
  const int no_l = g.no_l, no_k = g.no_k;
  int l1, k1, l2, k2;
  switch (ind) {
    case 1: l1 = 1; k1 = 1; l2 = 1; k2 = no_k; break;
    case 2: l1 = 1; k1 = no_k; l2 = no_l; k2 = no_k; break;
    case 3: l1 = no_l; k1 = no_k; l2 = no_l; k2 = 1; break;
    default: l1 = no_l; k1 = 1; l2 = 1; k2 = 1; break;
  }
  const double s1 = point[0], r1 = point[1], s2 = point[2], r2 = point[3];
  double w1 = point[4], w2 = point[5];
  const int kmin = std::min(k1, k2), kmax = std::max(k1, k2);
  const int lmin = std::min(l1, l2), lmax = std::max(l1, l2);
  const double dr = r2 - r1, ds = s2 - s1;
  const int il = std::max(1, lmax - lmin), ik = std::max(1, kmax - kmin);
  const double fac = w1 + w2;
  bool weighted = false;
  if (fac > zerocut) {
    weighted = true;
    w1 = w1 / fac;
    w2 = w2 / fac;
    if (rtyp == 4)
      throw DeckError("ERROR: consistency between user weights and line weights not yet coded");
  }
  if (lmin == lmax) {
    const double dd = (double)ik;
    for (int kk = kmin; kk <= kmax; kk++) {
      const int ki = kmin == k2 ? kmax + kmin - kk : kk;
      g.r(l1 - 1, ki - 1) = r1 + (double)(kk - kmin) * dr / dd;
      g.s(l1 - 1, ki - 1) = s1 + (double)(kk - kmin) * ds / dd;
      g.b(l1 - 1, ki - 1) = segbc;
    }
    if (weighted) {
      while (true) {
        bool done = true;
        for (int kk = kmin + 1; kk < kmax; kk++) {
          const double d_r = w1 * g.r(l1 - 1, kk - 2) + w2 * g.r(l1 - 1, kk) - g.r(l1 - 1, kk - 1);
          const double d_s = w1 * g.s(l1 - 1, kk - 2) + w2 * g.s(l1 - 1, kk) - g.s(l1 - 1, kk - 1);
          if (std::fabs(d_r) > tol || std::fabs(d_s) > tol) done = false;
          g.r(l1 - 1, kk - 1) += om * d_r;
          g.s(l1 - 1, kk - 1) += om * d_s;
        }
        if (done) break;
      }
    }
  } else {
    const double dd = (double)il;
    for (int ll = lmin; ll <= lmax; ll++) {
      const int li = lmin == l2 ? lmax + lmin - ll : ll;
      g.r(li - 1, k1 - 1) = r1 + (double)(ll - lmin) * dr / dd;
      g.s(li - 1, k1 - 1) = s1 + (double)(ll - lmin) * ds / dd;
      g.b(li - 1, k1 - 1) = segbc;
    }
    if (weighted) {
      while (true) {
        bool done = true;
        for (int ll = lmin + 1; ll < lmax; ll++) {
          const double d_r = w1 * g.r(ll - 2, k1 - 1) + w2 * g.r(ll, k1 - 1) - g.r(ll - 1, k1 - 1);
          const double d_s = w1 * g.s(ll - 2, k1 - 1) + w2 * g.s(ll, k1 - 1) - g.s(ll - 1, k1 - 1);
          if (std::fabs(d_r) > tol || std::fabs(d_s) > tol) done = false;
          g.r(ll - 1, k1 - 1) += om * d_r;
          g.s(ll - 1, k1 - 1) += om * d_s;
        }
        if (done) break;
      }
    }
  }
}

constexpr double kPi = 3.1415926535897932385;
constexpr double kTwoPi = 6.2831853071795864770;

// polar angle of the offset (d along s, w along r) from an arc's centre as
// setup_mesh_arc measures it: atan(d/w), moved by pi where w < 0 and by
// 2 pi where only d < 0 (w near zero taken as zerocut)
double arc_angle(double d, double w, double zerocut) {
  const double den = std::fabs(w) < zerocut ? zerocut : w;
  double th = std::atan(d / den);
  if (den < 0.0) th = th + kPi;
  else if (d < 0.0) th = th + kTwoPi;
  return th;
}

// setup_mesh_arc (setup_mesh.F90:1857-2062) for one side: points at equal
// steps of polar angle about (s0, r0) = (point(6), point(5)) from the
// segment's first point to its second, radius linear in the angle; ARC_A
// runs anticlockwise, ARC_C is generated from its second point to its
// first and then reversed.  With weights (point(7:8)) the angles are
// relaxed first; that form is restated as written, including its use of
// the relaxation's last residual as the start radius and of r0 as the s
// offset.
void side_arc(Grid& g, const double* point, int segbc, int sty, int ind, double zerocut,
              double tol) {
  const int no_l = g.no_l, no_k = g.no_k;
  int l1, k1, l2, k2;
  switch (ind) {
    case 1: l1 = 1; k1 = 1; l2 = 1; k2 = no_k; break;
    case 2: l1 = 1; k1 = no_k; l2 = no_l; k2 = no_k; break;
    case 3: l1 = no_l; k1 = no_k; l2 = no_l; k2 = 1; break;
    default: l1 = no_l; k1 = 1; l2 = 1; k2 = 1; break;
  }
  const bool fl = sty == 2;
  const double s1 = fl ? point[2] : point[0], r1 = fl ? point[3] : point[1];
  const double s2 = fl ? point[0] : point[2], r2 = fl ? point[1] : point[3];
  const double r0 = point[4], s0 = point[5];
  double w1 = point[6], w2 = point[7];
  const int kmin = std::min(k1, k2), kmax = std::max(k1, k2);
  const int lmin = std::min(l1, l2), lmax = std::max(l1, l2);
  const double fac = w1 + w2;
  bool weighted = false;
  if (fac > zerocut) {
    w1 = w1 / fac;
    w2 = w2 / fac;
    weighted = true;
  }
  const double dd = s1 - s0, w3 = r1 - r0;
  const double theta1 = arc_angle(dd, w3, zerocut);
  double d1 = s2 - s0;
  const double w4 = r2 - r0;
  double theta2 = arc_angle(d1, w4, zerocut);
  if (theta2 > theta1) theta2 = theta2 - kTwoPi;
  const double d2 = std::sqrt(w4 * w4 + d1 * d1);
  d1 = std::sqrt(w3 * w3 + dd * dd);
  const bool along_k = lmin == lmax;
  const int lo = along_k ? kmin : lmin, hi = along_k ? kmax : lmax;
  const int end2 = along_k ? k2 : l2;
  auto R = [&](int i) -> double& { return along_k ? g.r(l1 - 1, i - 1) : g.r(i - 1, k1 - 1); };
  auto S = [&](int i) -> double& { return along_k ? g.s(l1 - 1, i - 1) : g.s(i - 1, k1 - 1); };
  auto B = [&](int i) -> int& { return along_k ? g.b(l1 - 1, i - 1) : g.b(i - 1, k1 - 1); };
  const double nd = (double)(hi - lo);
  const double dtheta = theta1 - theta2;
  for (int ii = lo; ii <= hi; ii++) {
    const int ij = lo == end2 ? hi + lo - ii : ii;
    const double theta = theta1 - (double)(ii - lo) * dtheta / nd;
    double dl = (d1 - d2) / dtheta;
    dl = d1 + dl * (theta - theta1);
    R(ij) = r0 + dl * std::cos(theta);
    S(ij) = s0 + dl * std::sin(theta);
    B(ij) = segbc;
  }
  g.r(l1 - 1, k1 - 1) = r1;
  g.r(l2 - 1, k2 - 1) = r2;
  g.s(l1 - 1, k1 - 1) = s1;
  g.s(l2 - 1, k2 - 1) = s2;
  if (weighted) {
    for (int ii = lo; ii <= hi; ii++) {
      const int ij = lo == end2 ? hi + lo - ii : ii;
      R(ij) = theta1 - (double)(ii - lo) * dtheta / nd;
    }
    while (true) {
      bool done = true;
      for (int ii = lo + 1; ii < hi; ii++) {
        d1 = w1 * R(ii - 1) + w2 * R(ii + 1) - R(ii);
        if (std::fabs(d1) > tol) done = false;
        R(ii) = R(ii) + d1;
      }
      if (done) break;
    }
    for (int ii = lo + 1; ii < hi; ii++) {
      const double theta = R(ii);
      double dl = (d1 - d2) / dtheta;
      dl = d1 + dl * (theta - theta1);
      R(ii) = r0 + dl * std::cos(theta);
      S(ii) = r0 + dl * std::sin(theta);
    }
  }
  if (fl) {
    for (int jj = 0; jj <= (hi - lo) / 2; jj++) {
      std::swap(R(lo + jj), R(hi - jj));
      std::swap(S(lo + jj), S(hi - jj));
    }
  }
}

// residual of the relaxation stencil (setup_mesh.F90:851-860) at an interior
// point, left to right like the reference
double stencil(Grid& g, bool r, const double* w, int l, int k) {
  auto x = [&](int a, int b) -> double { return r ? g.r(a, b) : g.s(a, b); };
  double d = w[0] * x(l + 1, k - 1);
  d = d + w[1] * x(l + 1, k);
  d = d + w[2] * x(l + 1, k + 1);
  d = d + w[3] * x(l, k - 1);
  d = d + w[4] * x(l, k + 1);
  d = d + w[5] * x(l - 1, k - 1);
  d = d + w[6] * x(l - 1, k);
  d = d + w[7] * x(l - 1, k + 1);
  return d - x(l, k);
}

void gauss_seidel(Grid& g, const double* rw, const double* sw, double tol, double om,
                  long max_it) {
  long it = 0;
  while (true) {
    it++;
    bool done = true;
    for (int kk = 1; kk < g.no_k - 1; kk++)
      for (int ll = 1; ll < g.no_l - 1; ll++) {
        const double d_r = rw[0] * g.r(ll + 1, kk - 1) + rw[1] * g.r(ll + 1, kk) +
                           rw[2] * g.r(ll + 1, kk + 1) + rw[3] * g.r(ll, kk - 1) +
                           rw[4] * g.r(ll, kk + 1) + rw[5] * g.r(ll - 1, kk - 1) +
                           rw[6] * g.r(ll - 1, kk) + rw[7] * g.r(ll - 1, kk + 1) - g.r(ll, kk);
        const double d_s = sw[0] * g.s(ll + 1, kk - 1) + sw[1] * g.s(ll + 1, kk) +
                           sw[2] * g.s(ll + 1, kk + 1) + sw[3] * g.s(ll, kk - 1) +
                           sw[4] * g.s(ll, kk + 1) + sw[5] * g.s(ll - 1, kk - 1) +
                           sw[6] * g.s(ll - 1, kk) + sw[7] * g.s(ll - 1, kk + 1) - g.s(ll, kk);
        if (std::fabs(d_r) > tol || std::fabs(d_s) > tol) {
          done = false;
          g.r(ll, kk) += om * d_r;
          g.s(ll, kk) += om * d_s;
        }
      }
    if (it > max_it || done) return;
  }
}

// one corner of setup_mesh.F90:885-1079 (a, b: the two edge neighbours)
void corner_bc(Grid& g, int l, int k, int a, int b) {
  auto is = [&](int x, int y) { return (a == x && b == y) || (a == y && b == x); };
  if (is(1, 2)) g.b(l, k) = 3;
  if (is(6, 1)) g.b(l, k) = 4;
  if (is(6, 2)) g.b(l, k) = 5;
  if (is(8, 1)) g.b(l, k) = 1;
  if (is(8, 2)) g.b(l, k) = 2;
  if (is(8, 3)) g.b(l, k) = 3;
  if (is(6, 3)) throw DeckError("ERROR: inconsistent BC at corner");
}

}  // namespace

MeshData generate_mesh(const Namelist* mesh_nl, double zerocut) {
  if (!mesh_nl) throw DeckError("ERROR: no MESH namelist");
  const Namelist& nl = *mesh_nl;
  const auto rtyp = nl.get_array("region_typ", {LI}, Value::str("    "));
  int nreg = 0;
  for (const auto& t : rtyp)
    if (!t.as_str().empty()) nreg++;
  if (nreg != 1) throw DeckError("ERROR: only single-region meshes are supported");
  const std::string t = rtyp[0].as_str();
  int typ;
  if (t == "LIN1") typ = 1;
  else if (t == "LIN2") typ = 2;
  else if (t == "EQUI") typ = 3;
  else if (t == "USER") typ = 4;
  else throw DeckError("ERROR: unrecognised region type");
  if (typ != 1 && typ != 2) throw DeckError("ERROR: region type " + t + " not supported");
  const auto rdim = nl.get_array("region_dim", {LI, 2}, Value::integer(0));
  const int dim1 = (int)rdim[1].as_int();  // reg%dim(1)=region_dim(i,2) (l)
  const int dim2 = (int)rdim[0].as_int();  // reg%dim(2)=region_dim(i,1) (k)
  if (dim1 <= 0) throw DeckError("ERROR: region L dimension <= 0");
  if (dim2 <= 0) throw DeckError("ERROR: region K dimension <=0");
  const double tol = nl.get_array("region_tol", {LI}, Value::real(1.0e-12))[0].as_real();
  const double om = nl.get_array("region_om", {LI}, Value::real(1.0))[0].as_real();
  const int mat = (int)nl.get_array("region_material", {LI}, Value::integer(0))[0].as_int();
  const auto side = nl.get_array("region_side", {LI, 4, LI}, Value::integer(0));
  const auto segtyp = nl.get_array("segment_typ", {LI}, Value::str("     "));
  const auto segbc = nl.get_array("segment_bc", {LI}, Value::str("FREE"));
  const auto segpos = nl.get_array("segment_pos", {LI, 8}, Value::real(0.0));
  Grid g;
  g.no_l = dim1 + 1;
  g.no_k = dim2 + 1;
  const int no_l = g.no_l, no_k = g.no_k;
  g.rr.assign((size_t)no_l * no_k, 0.0);
  g.ss.assign((size_t)no_l * no_k, 0.0);
  g.bc.assign((size_t)no_l * no_k, 0);
  double rw[8] = {0}, sw[8] = {0};
  if (typ == 1) {
    rw[1] = rw[6] = sw[1] = sw[6] = 1.0;
  } else {
    rw[3] = rw[4] = sw[3] = sw[4] = 1.0;
  }
  {
    double tl0 = 0, tl1 = 0;
    for (int q = 0; q < 8; q++) {
      tl0 += rw[q];
      tl1 += sw[q];
    }
    for (int q = 0; q < 8; q++) {
      rw[q] = rw[q] / tl0;
      sw[q] = sw[q] / tl1;
    }
  }
  for (int ind = 1; ind <= 4; ind++) {
    // region_side(1, ind, 1) = number of segments, (1, ind, 2) = the segment
    const int nseg = (int)side[(size_t)(ind - 1) * LI + 0].as_int();
    if (nseg != 1) throw DeckError("ERROR: only one segment per region side is supported");
    const int iseg = (int)side[(size_t)(ind - 1) * LI + 1].as_int();
    if (iseg < 1 || iseg > LI) throw DeckError("ERROR: bad segment index");
    const std::string st = segtyp[iseg - 1].as_str();
    int sty;
    if (st == "LINE") sty = 1;
    else if (st == "ARC_C") sty = 2;
    else if (st == "ARC_A") sty = 3;
    else if (st == "POINT") sty = 4;
    else if (st == "LINK") sty = 5;
    else throw DeckError("ERROR: unrecognised segment type");
    if (sty == 4) throw DeckError("ERROR: side_type is POINT but DJN off");
    const int b = bc_code(segbc[iseg - 1].as_str());
    double point[8];
    for (int q = 0; q < 8; q++) point[q] = segpos[(size_t)(iseg - 1) * 8 + q].as_real();
    if (sty == 2 || sty == 3)
      side_arc(g, point, b, sty, ind, zerocut, tol);
    else
      side_line(g, point, b, ind, zerocut, tol, om, typ);
  }
  // interior initial guess (setup_mesh.F90:713-752)
  const int l1 = 2, k1 = 2, l2 = no_l - 1, k2 = no_k - 1;
  double tl0 = rw[6], tl1 = rw[1], tk0 = rw[3], tk1 = rw[4];
  double fac = tl0 + tl1 + tk0 + tk1;
  if (std::fabs(fac) <= zerocut) fac = 1.0;
  tl0 = 2.0 * tl0 / fac;
  tl1 = 2.0 * tl1 / fac;
  tk0 = 2.0 * tk0 / fac;
  tk1 = 2.0 * tk1 / fac;
  if (l2 >= l1 && k2 >= k1) {
    for (int pass = 0; pass < 2; pass++) {
      const bool r = pass == 0;
      // all points use the side values only, so the order does not matter
      for (int ll = l1; ll <= l2; ll++)
        for (int kk = k1; kk <= k2; kk++) {
          double ww = (double)(l2 - l1) + 2.0;
          const double wl0 = tl0 * (((double)l2 - (double)ll) + 1.0) / ww;
          const double wl1 = tl1 * (((double)ll - (double)l1) + 1.0) / ww;
          ww = (double)(k2 - k1) + 2.0;
          const double wk0 = tk0 * (((double)k2 - (double)kk) + 1.0) / ww;
          const double wk1 = tk1 * (((double)kk - (double)k1) + 1.0) / ww;
          auto a = [&](int l, int k) -> double { return r ? g.r(l, k) : g.s(l, k); };
          const double v = ((wk0 * a(ll - 1, k1 - 2) + wk1 * a(ll - 1, k2)) + wl0 * a(l1 - 2, kk - 1)) +
                           wl1 * a(l2, kk - 1);
          if (r) g.r(ll - 1, kk - 1) = v;
          else g.s(ll - 1, kk - 1) = v;
        }
    }
    // relaxation (setup_mesh.F90:795-877): one sweep, the Gauss-Seidel
    // iteration only if a point actually moves
    bool moves = false;
    for (int ll = 1; ll < no_l - 1 && !moves; ll++)
      for (int kk = 1; kk < no_k - 1; kk++)
        if (std::fabs(stencil(g, true, rw, ll, kk)) > tol ||
            std::fabs(stencil(g, false, sw, ll, kk)) > tol) {
          moves = true;
          break;
        }
    if (moves) gauss_seidel(g, rw, sw, tol, om, 8L * no_l * no_k);
  }
  // corner boundary conditions (setup_mesh.F90:885-1079)
  corner_bc(g, 0, 0, g.b(1, 0), g.b(0, 1));
  corner_bc(g, 0, no_k - 1, g.b(1, no_k - 1), g.b(0, no_k - 2));
  corner_bc(g, no_l - 1, 0, g.b(no_l - 2, 0), g.b(no_l - 1, 1));
  corner_bc(g, no_l - 1, no_k - 1, g.b(no_l - 2, no_k - 1), g.b(no_l - 1, no_k - 2));
  // setup_mesh_transfer (setup_mesh.F90:1091-1250): node (l,k) ->
  // l + (k-1)*no_l, x = s, y = r
  MeshData m;
  const int nnd = no_l * no_k;
  m.ndx.resize(nnd);
  m.ndy.resize(nnd);
  m.indtype.resize(nnd);
  for (int kk = 0; kk < no_k; kk++)
    for (int ll = 0; ll < no_l; ll++) {
      const int n = ll + kk * no_l;
      m.ndx[n] = g.s(ll, kk);
      m.ndy[n] = g.r(ll, kk);
      const bool edge = kk == 0 || kk == no_k - 1 || ll == 0 || ll == no_l - 1;
      const int b = g.b(ll, kk);
      if (edge && b <= 0) throw DeckError("ERROR: undefined BC at region edge");
      m.indtype[n] = edge ? -b : 1;
    }
  // orientation test (setup_mesh.F90:1202-1215)
  const double r1 = g.r(1, 0) - g.r(0, 0), r2 = g.r(0, 1) - g.r(0, 0), r3 = g.r(1, 1) - g.r(0, 0);
  const double s1 = g.s(1, 0) - g.s(0, 0), s2 = g.s(0, 1) - g.s(0, 0), s3 = g.s(1, 1) - g.s(0, 0);
  int i1 = 1, i2 = 3;
  if ((r1 * s2 - r2 * s1) > 0.0 || (r1 * s3 - r3 * s1) > 0.0 || (r3 * s2 - r2 * s3) > 0.0) {
    i1 = 3;
    i2 = 1;
  }
  const int nel = (no_l - 1) * (no_k - 1);
  m.ielnd.resize((size_t)nel * 4);
  int e = 0;
  for (int kk = 1; kk < no_k; kk++)
    for (int ll = 1; ll < no_l; ll++, e++) {
      int* c = &m.ielnd[(size_t)e * 4];
      c[0] = ll + (kk - 1) * no_l;
      c[2] = (ll + 1) + kk * no_l;
      c[i1] = c[0] + 1;
      c[i2] = c[2] - 1;
    }
  m.ielreg.assign(nel, 1);
  m.ielmat.assign(nel, mat);
  m.nel = nel;
  m.nnd = nnd;
  connectivity(m.ielnd, nel, m.ielel, m.ielfc);
  nodetype(m.ielnd, nel, m.indtype);
  return m;
}

void connectivity(const std::vector<int>& ielnd, int nel, std::vector<int>& ielel,
                  std::vector<int>& ielfc) {
  // faces j: corner j -> j+1; a shared face appears twice with the same
  // (low, high) node pair
  struct F {
    long long lo, hi;
    int f;
  };
  std::vector<F> fs((size_t)nel * 4);
  for (int e = 0; e < nel; e++)
    for (int j = 0; j < 4; j++) {
      const long long a = ielnd[(size_t)e * 4 + j], b = ielnd[(size_t)e * 4 + ((j + 1) & 3)];
      fs[(size_t)e * 4 + j] = {std::min(a, b), std::max(a, b), e * 4 + j};
    }
  std::stable_sort(fs.begin(), fs.end(), [](const F& x, const F& y) {
    return x.lo != y.lo ? x.lo < y.lo : x.hi < y.hi;
  });
  ielel.assign((size_t)nel * 4, 0);
  ielfc.assign((size_t)nel * 4, 0);
  for (size_t p = 0; p + 1 < fs.size(); p++) {
    if (fs[p].lo == fs[p + 1].lo && fs[p].hi == fs[p + 1].hi) {
      const int fa = fs[p].f, fb = fs[p + 1].f;
      ielel[fa] = fb / 4 + 1;
      ielel[fb] = fa / 4 + 1;
      ielfc[fa] = fb % 4 + 1;
      ielfc[fb] = fa % 4 + 1;
    }
  }
  // corrconn: boundary faces point at themselves, side = opposite face
  for (int j1 = 0; j1 < 2; j1++) {
    const int j2 = j1 + 2;
    for (int e = 0; e < nel; e++) {
      if (ielel[(size_t)e * 4 + j1] == 0) {
        ielel[(size_t)e * 4 + j1] = e + 1;
        ielfc[(size_t)e * 4 + j1] = j2 + 1;
      }
      if (ielel[(size_t)e * 4 + j2] == 0) {
        ielel[(size_t)e * 4 + j2] = e + 1;
        ielfc[(size_t)e * 4 + j2] = j1 + 1;
      }
    }
  }
}

void nodetype(const std::vector<int>& ielnd, int nel, std::vector<int>& indtype) {
  const int nnd = (int)indtype.size();
  for (int e = 0; e < nel; e++) {
    const int* nodes = &ielnd[(size_t)e * 4];
    int neg = 0;
    for (int j = 0; j < 4; j++) neg += indtype[nodes[j] - 1] < 0 ? 1 : 0;
    if (neg != 3) continue;
    int ii = 0;
    while (ii < 4 && !(indtype[nodes[ii] - 1] > 0)) ii++;
    ii = (ii + 2) % 4;
    const int jj = nodes[ii];
    if (jj <= nnd) {
      const int t1 = indtype[nodes[(ii + 1) % 4] - 1], t2 = indtype[nodes[(ii + 3) % 4] - 1];
      if ((t1 == -2 && t2 == -1) || (t2 == -2 && t1 == -1)) indtype[jj - 1] = -3;
    }
  }
}

}  // namespace blh
