"""Structured-region mesh generator, numbering, connectivity and node types.

Host-side restatement of the reference's setup (out of the GPU hot path):

  setup_mesh_read_input   setup_mesh.F90:106-346   (MESH namelist)
  setup_mesh_region       setup_mesh.F90:593-1089  (LIN1/LIN2 weights, side
                                                    lines, interior guess and
                                                    relaxation, corner BCs)
  setup_mesh_line         setup_mesh.F90:1750-1855
  setup_mesh_arc          setup_mesh.F90:1857-2062
  setup_mesh_transfer     setup_mesh.F90:1091-1250 (node/element numbering)
  utils_kn_getconn/getsconn/corrconn   utils_kn_connectivity.f90:30-170
  init_kn_nodetype        init_kn.f90:78-106

Supported: one mesh region of type LIN1 or LIN2 whose four sides are single
LINE, LINK, ARC_A or ARC_C segments -- every deck in the reference's
input/ directory.  Node ``l`` runs along region_dim(:,2),
``k`` along region_dim(:,1), exactly as the reference stores them, so node and
element numbers match the reference's.
"""
import numpy as np

from .deck import DeckError, LI, Namelist

BC_CODES = {"SLIPX": 1, "SLIPY": 2, "WALL": 3, "TRANS": 6, "OPEN": 7, "FREE": 8}
SEG_TYPES = {"LINE": 1, "ARC_C": 2, "ARC_A": 3, "POINT": 4, "LINK": 5}
REG_TYPES = {"LIN1": 1, "LIN2": 2, "EQUI": 3, "USER": 4}


class Mesh:
    """Single-partition mesh in the reference's numbering (1-based ids)."""

    def __init__(self, ndx, ndy, indtype, ielnd, ielreg, ielmat):
        self.ndx = ndx
        self.ndy = ndy
        self.indtype = indtype
        self.ielnd = ielnd          # (nel, 4) int32, 1-based node ids
        self.ielreg = ielreg
        self.ielmat = ielmat
        self.nel = ielnd.shape[0]
        self.nnd = ndx.shape[0]
        self.ielel, self.ielfc = connectivity(ielnd)
        nodetype(self.ielnd, self.indtype)


def _side_line(rr, ss, bc, seg, ind, no_l, no_k, zerocut, tol, om, rtyp):
    """setup_mesh_line (setup_mesh.F90:1750-1855) for one side."""
    l1, k1, l2, k2 = {1: (1, 1, 1, no_k), 2: (1, no_k, no_l, no_k),
                      3: (no_l, no_k, no_l, 1), 4: (no_l, 1, 1, 1)}[ind]
    s1, r1, s2, r2, w1, w2 = seg["point"][:6]
    kmin, kmax = min(k1, k2), max(k1, k2)
    lmin, lmax = min(l1, l2), max(l1, l2)
    dr = r2 - r1
    ds = s2 - s1
    il = max(1, lmax - lmin)
    ik = max(1, kmax - kmin)
    fac = w1 + w2
    weighted = False
    if fac > zerocut:
        weighted = True
        w1 = w1 / fac
        w2 = w2 / fac
        if rtyp == 4:
            raise DeckError("ERROR: consistency between user weights and line weights not yet coded")
    if lmin == lmax:
        dd = float(ik)
        for kk in range(kmin, kmax + 1):
            ki = kmax + kmin - kk if kmin == k2 else kk
            rr[l1 - 1, ki - 1] = r1 + float(kk - kmin) * dr / dd
            ss[l1 - 1, ki - 1] = s1 + float(kk - kmin) * ds / dd
            bc[l1 - 1, ki - 1] = seg["bc"]
        if weighted:
            while True:
                done = True
                for kk in range(kmin + 1, kmax):
                    d_r = w1 * rr[l1 - 1, kk - 2] + w2 * rr[l1 - 1, kk] - rr[l1 - 1, kk - 1]
                    d_s = w1 * ss[l1 - 1, kk - 2] + w2 * ss[l1 - 1, kk] - ss[l1 - 1, kk - 1]
                    if abs(d_r) > tol or abs(d_s) > tol:
                        done = False
                    rr[l1 - 1, kk - 1] += om * d_r
                    ss[l1 - 1, kk - 1] += om * d_s
                if done:
                    break
    else:
        dd = float(il)
        for ll in range(lmin, lmax + 1):
            li = lmax + lmin - ll if lmin == l2 else ll
            rr[li - 1, k1 - 1] = r1 + float(ll - lmin) * dr / dd
            ss[li - 1, k1 - 1] = s1 + float(ll - lmin) * ds / dd
            bc[li - 1, k1 - 1] = seg["bc"]
        if weighted:
            while True:
                done = True
                for ll in range(lmin + 1, lmax):
                    d_r = w1 * rr[ll - 2, k1 - 1] + w2 * rr[ll, k1 - 1] - rr[ll - 1, k1 - 1]
                    d_s = w1 * ss[ll - 2, k1 - 1] + w2 * ss[ll, k1 - 1] - ss[ll - 1, k1 - 1]
                    if abs(d_r) > tol or abs(d_s) > tol:
                        done = False
                    rr[ll - 1, k1 - 1] += om * d_r
                    ss[ll - 1, k1 - 1] += om * d_s
                if done:
                    break


PI = 3.1415926535897932385
TWOPI = 6.2831853071795864770


def _arc_angle(d, w, zerocut):
    """Polar angle of the offset (d along s, w along r) from the arc's
    centre, in [0, 2 pi) as setup_mesh_arc measures it: atan(d / w) moved by
    pi where w < 0 and by 2 pi where only d < 0 (w near zero taken as
    zerocut)."""
    import math
    den = zerocut if abs(w) < zerocut else w
    th = math.atan(d / den)
    if den < 0.0:
        th = th + PI
    elif d < 0.0:
        th = th + TWOPI
    return th


def _side_arc(rr, ss, bc, seg, ind, no_l, no_k, zerocut, tol, om):
    """setup_mesh_arc (setup_mesh.F90:1857-2062) for one side: points at
    equal steps of polar angle about (s0, r0) = (point(6), point(5)) from
    the segment's first point to its second, with the radius interpolated
    linearly in the angle; ARC_A runs anticlockwise, ARC_C is generated
    from its second point to its first and then reversed.  With weights
    (point(7:8)) the angles are relaxed first.  Restated as written,
    including two quirks of the weighted form: the radius slope there uses
    the relaxation's last residual in place of the start radius, and the
    s coordinate is offset by r0."""
    import math
    l1, k1, l2, k2 = {1: (1, 1, 1, no_k), 2: (1, no_k, no_l, no_k),
                      3: (no_l, no_k, no_l, 1), 4: (no_l, 1, 1, 1)}[ind]
    p = seg["point"]
    fl = seg["typ"] == 2
    if fl:
        s1, r1, s2, r2 = p[2], p[3], p[0], p[1]
    else:
        s1, r1, s2, r2 = p[0], p[1], p[2], p[3]
    r0, s0, w1, w2 = p[4], p[5], p[6], p[7]
    kmin, kmax = min(k1, k2), max(k1, k2)
    lmin, lmax = min(l1, l2), max(l1, l2)
    fac = w1 + w2
    weighted = False
    if fac > zerocut:
        w1 = w1 / fac
        w2 = w2 / fac
        weighted = True
    dd = s1 - s0
    w3 = r1 - r0
    theta1 = _arc_angle(dd, w3, zerocut)
    d1 = s2 - s0
    w4 = r2 - r0
    theta2 = _arc_angle(d1, w4, zerocut)
    if theta2 > theta1:
        theta2 = theta2 - TWOPI
    d2 = math.sqrt(w4 * w4 + d1 * d1)
    d1 = math.sqrt(w3 * w3 + dd * dd)
    along_k = lmin == lmax
    lo, hi = (kmin, kmax) if along_k else (lmin, lmax)
    end2 = k2 if along_k else l2

    def at(i):          # (l, k) 0-based index of position i along the side
        return (l1 - 1, i - 1) if along_k else (i - 1, k1 - 1)

    nd = float(hi - lo)
    dtheta = theta1 - theta2
    for ii in range(lo, hi + 1):
        ij = hi + lo - ii if lo == end2 else ii
        theta = theta1 - float(ii - lo) * dtheta / nd
        dl = (d1 - d2) / dtheta
        dl = d1 + dl * (theta - theta1)
        rr[at(ij)] = r0 + dl * math.cos(theta)
        ss[at(ij)] = s0 + dl * math.sin(theta)
        bc[at(ij)] = seg["bc"]
    rr[l1 - 1, k1 - 1] = r1
    rr[l2 - 1, k2 - 1] = r2
    ss[l1 - 1, k1 - 1] = s1
    ss[l2 - 1, k2 - 1] = s2
    if weighted:
        for ii in range(lo, hi + 1):
            ij = hi + lo - ii if lo == end2 else ii
            rr[at(ij)] = theta1 - float(ii - lo) * dtheta / nd
        while True:
            done = True
            for ii in range(lo + 1, hi):
                d1 = w1 * rr[at(ii - 1)] + w2 * rr[at(ii + 1)] - rr[at(ii)]
                if abs(d1) > tol:
                    done = False
                rr[at(ii)] = rr[at(ii)] + d1
            if done:
                break
        for ii in range(lo + 1, hi):
            theta = rr[at(ii)]
            dl = (d1 - d2) / dtheta
            dl = d1 + dl * (theta - theta1)
            rr[at(ii)] = r0 + dl * math.cos(theta)
            ss[at(ii)] = r0 + dl * math.sin(theta)
    if fl:
        for jj in range(0, (hi - lo) // 2 + 1):
            a, b = at(lo + jj), at(hi - jj)
            rr[a], rr[b] = rr[b], rr[a]
            ss[a], ss[b] = ss[b], ss[a]


def _stencil(x, w):
    """Residual of the relaxation stencil (setup_mesh.F90:851-860) at every
    interior point, evaluated left to right like the reference."""
    lp = slice(2, None)
    lm = slice(0, -2)
    mid = slice(1, -1)
    # r1*x(lp,km)+r2*x(lp,kk)+r3*x(lp,kp)+r4*x(ll,km)+r5*x(ll,kp)+
    # r6*x(lm,km)+r7*x(lm,kk)+r8*x(lm,kp)-x(ll,kk), left to right
    d = w[0] * x[lp, lm]
    d = d + w[1] * x[lp, mid]
    d = d + w[2] * x[lp, lp]
    d = d + w[3] * x[mid, lm]
    d = d + w[4] * x[mid, lp]
    d = d + w[5] * x[lm, lm]
    d = d + w[6] * x[lm, mid]
    d = d + w[7] * x[lm, lp]
    return d - x[mid, mid]


def generate(mesh_nl, zerocut):
    """Return (ndx, ndy, indtype, ielnd, ielreg_mesh, reg_mat) for the MESH
    namelist of a control file (setup_mesh_gen)."""
    if not isinstance(mesh_nl, Namelist):
        raise DeckError("ERROR: no MESH namelist")
    rtyp = mesh_nl.get_array("region_typ", (LI,), "    ")
    nreg = sum(1 for t in rtyp if str(t).strip())
    if nreg != 1:
        raise DeckError("ERROR: only single-region meshes are supported")
    t = str(rtyp[0]).strip().upper()
    if t not in REG_TYPES:
        raise DeckError("ERROR: unrecognised region type")
    typ = REG_TYPES[t]
    if typ not in (1, 2):
        raise DeckError("ERROR: region type %s not supported" % t)
    rdim = mesh_nl.get_array("region_dim", (LI, 2), 0)
    dim1 = int(rdim[0, 1])     # reg%dim(1)=region_dim(i,2)  (l direction)
    dim2 = int(rdim[0, 0])     # reg%dim(2)=region_dim(i,1)  (k direction)
    if dim1 <= 0:
        raise DeckError("ERROR: region L dimension <= 0")
    if dim2 <= 0:
        raise DeckError("ERROR: region K dimension <=0")
    tol = float(mesh_nl.get_array("region_tol", (LI,), 1.0e-12)[0])
    om = float(mesh_nl.get_array("region_om", (LI,), 1.0)[0])
    mat = int(mesh_nl.get_array("region_material", (LI,), 0)[0])
    side = mesh_nl.get_array("region_side", (LI, 4, LI), 0)
    segtyp = mesh_nl.get_array("segment_typ", (LI,), "     ")
    segbc = mesh_nl.get_array("segment_bc", (LI,), "FREE")
    segpos = mesh_nl.get_array("segment_pos", (LI, 8), 0.0)
    no_l, no_k = dim1 + 1, dim2 + 1
    rr = np.zeros((no_l, no_k))
    ss = np.zeros((no_l, no_k))
    bc = np.zeros((no_l, no_k), dtype=np.int32)
    rw = np.zeros(8)
    sw = np.zeros(8)
    if typ == 1:
        rw[1] = rw[6] = sw[1] = sw[6] = 1.0
    else:
        rw[3] = rw[4] = sw[3] = sw[4] = 1.0
    tl0, tl1 = rw.sum(), sw.sum()
    rw = rw / tl0
    sw = sw / tl1
    for ind in range(1, 5):
        nseg = int(side[0, ind - 1, 0])
        if nseg != 1:
            raise DeckError("ERROR: only one segment per region side is supported")
        iseg = int(side[0, ind - 1, 1])
        st = str(segtyp[iseg - 1]).strip().upper()
        if st not in SEG_TYPES:
            raise DeckError("ERROR: unrecognised segment type")
        if SEG_TYPES[st] == 4:
            raise DeckError("ERROR: side_type is POINT but DJN off")
        b = str(segbc[iseg - 1]).strip().upper()
        if b not in BC_CODES:
            raise DeckError("ERROR: unrecognised segment boundary condition")
        seg = {"point": [float(v) for v in segpos[iseg - 1, :]], "bc": BC_CODES[b],
               "typ": SEG_TYPES[st]}
        if SEG_TYPES[st] in (2, 3):
            _side_arc(rr, ss, bc, seg, ind, no_l, no_k, zerocut, tol, om)
        else:
            _side_line(rr, ss, bc, seg, ind, no_l, no_k, zerocut, tol, om, typ)
    # interior initial guess (setup_mesh.F90:713-752)
    l1, k1, l2, k2 = 2, 2, no_l - 1, no_k - 1
    tl0, tl1, tk0, tk1 = rw[6], rw[1], rw[3], rw[4]
    fac = tl0 + tl1 + tk0 + tk1
    if abs(fac) <= zerocut:
        fac = 1.0
    tl0 = 2.0 * tl0 / fac
    tl1 = 2.0 * tl1 / fac
    tk0 = 2.0 * tk0 / fac
    tk1 = 2.0 * tk1 / fac
    if l2 >= l1 and k2 >= k1:
        ll = np.arange(l1, l2 + 1, dtype=np.float64)[:, None]
        kk = np.arange(k1, k2 + 1, dtype=np.float64)[None, :]
        ww = float(l2 - l1) + 2.0
        wl0 = tl0 * ((float(l2) - ll) + 1.0) / ww
        wl1 = tl1 * ((ll - float(l1)) + 1.0) / ww
        ww = float(k2 - k1) + 2.0
        wk0 = tk0 * ((float(k2) - kk) + 1.0) / ww
        wk1 = tk1 * ((kk - float(k1)) + 1.0) / ww
        for a in (rr, ss):
            # wk0*a(ll,k1-1)+wk1*a(ll,k2+1)+wl0*a(l1-1,kk)+wl1*a(l2+1,kk)
            a[l1 - 1:l2, k1 - 1:k2] = (
                ((wk0 * a[l1 - 1:l2, [k1 - 2]] + wk1 * a[l1 - 1:l2, [k2]])
                 + wl0 * a[[l1 - 2], k1 - 1:k2]) + wl1 * a[[l2], k1 - 1:k2])
        # relaxation (setup_mesh.F90:795-877): one sweep, exact Gauss-Seidel
        # fallback only if a point actually moves
        dr = _stencil(rr, rw)
        ds = _stencil(ss, sw)
        if np.any((np.abs(dr) > tol) | (np.abs(ds) > tol)):
            _gauss_seidel(rr, ss, rw, sw, tol, om, 8 * no_l * no_k)
    # corner boundary conditions (setup_mesh.F90:885-1079)
    _corner_bc(bc, 0, 0, bc[1, 0], bc[0, 1])
    _corner_bc(bc, 0, no_k - 1, bc[1, no_k - 1], bc[0, no_k - 2])
    _corner_bc(bc, no_l - 1, 0, bc[no_l - 2, 0], bc[no_l - 1, 1])
    _corner_bc(bc, no_l - 1, no_k - 1, bc[no_l - 2, no_k - 1], bc[no_l - 1, no_k - 2])
    return _transfer(rr, ss, bc, no_l, no_k, mat)


def _gauss_seidel(rr, ss, rw, sw, tol, om, max_it):
    no_l, no_k = rr.shape
    it = 0
    while True:
        it += 1
        done = True
        for kk in range(1, no_k - 1):
            for ll in range(1, no_l - 1):
                d_r = (rw[0] * rr[ll + 1, kk - 1] + rw[1] * rr[ll + 1, kk] + rw[2] * rr[ll + 1, kk + 1]
                       + rw[3] * rr[ll, kk - 1] + rw[4] * rr[ll, kk + 1] + rw[5] * rr[ll - 1, kk - 1]
                       + rw[6] * rr[ll - 1, kk] + rw[7] * rr[ll - 1, kk + 1] - rr[ll, kk])
                d_s = (sw[0] * ss[ll + 1, kk - 1] + sw[1] * ss[ll + 1, kk] + sw[2] * ss[ll + 1, kk + 1]
                       + sw[3] * ss[ll, kk - 1] + sw[4] * ss[ll, kk + 1] + sw[5] * ss[ll - 1, kk - 1]
                       + sw[6] * ss[ll - 1, kk] + sw[7] * ss[ll - 1, kk + 1] - ss[ll, kk])
                if abs(d_r) > tol or abs(d_s) > tol:
                    done = False
                    rr[ll, kk] += om * d_r
                    ss[ll, kk] += om * d_s
        if it > max_it or done:
            return


def _corner_bc(bc, l, k, a, b):
    """One corner of setup_mesh.F90:885-1079 (a, b: the two edge neighbours)."""
    pair = {a, b}
    if pair == {1, 2}:
        bc[l, k] = 3
    if pair == {6, 1}:
        bc[l, k] = 4
    if pair == {6, 2}:
        bc[l, k] = 5
    if pair == {8, 1}:
        bc[l, k] = 1
    if pair == {8, 2}:
        bc[l, k] = 2
    if pair == {8, 3}:
        bc[l, k] = 3
    if pair == {6, 3}:
        raise DeckError("ERROR: inconsistent BC at corner")


def _transfer(rr, ss, bc, no_l, no_k, mat):
    """setup_mesh_transfer (setup_mesh.F90:1091-1250) for one region."""
    # node (ll,kk) -> ll + (kk-1)*no_l; x = ss, y = rr
    ndx = np.ascontiguousarray(ss.T).reshape(-1).copy()
    ndy = np.ascontiguousarray(rr.T).reshape(-1).copy()
    b = np.ascontiguousarray(bc.T).reshape(-1)
    edge = np.zeros((no_k, no_l), dtype=bool)
    edge[0, :] = edge[-1, :] = True
    edge[:, 0] = edge[:, -1] = True
    edge = edge.reshape(-1)
    if np.any(edge & (b <= 0)):
        raise DeckError("ERROR: undefined BC at region edge")
    indtype = np.where(edge, -b, 1).astype(np.int32)
    # orientation test (setup_mesh.F90:1202-1215)
    r1 = rr[1, 0] - rr[0, 0]
    r2 = rr[0, 1] - rr[0, 0]
    r3 = rr[1, 1] - rr[0, 0]
    s1 = ss[1, 0] - ss[0, 0]
    s2 = ss[0, 1] - ss[0, 0]
    s3 = ss[1, 1] - ss[0, 0]
    if (r1 * s2 - r2 * s1) > 0.0 or (r1 * s3 - r3 * s1) > 0.0 or (r3 * s2 - r2 * s3) > 0.0:
        i1, i2 = 3, 1
    else:
        i1, i2 = 1, 3
    kk, ll = np.meshgrid(np.arange(1, no_k), np.arange(1, no_l), indexing="ij")
    kk = kk.reshape(-1)
    ll = ll.reshape(-1)
    nel = kk.size
    ielnd = np.zeros((nel, 4), dtype=np.int32)
    ielnd[:, 0] = ll + (kk - 1) * no_l
    ielnd[:, 2] = (ll + 1) + kk * no_l
    ielnd[:, i1] = ielnd[:, 0] + 1
    ielnd[:, i2] = ielnd[:, 2] - 1
    ielreg = np.ones(nel, dtype=np.int32)
    ielmat = np.full(nel, mat, dtype=np.int32)
    return ndx, ndy, indtype, ielnd, ielreg, ielmat


def connectivity(ielnd):
    """ielel/ielfc from utils_kn_getconn + getsconn + corrconn
    (utils_kn_connectivity.f90:30-170), 1-based, boundary face -> self and
    the opposite face."""
    nel = ielnd.shape[0]
    a = ielnd.astype(np.int64)
    n1 = a
    n2 = np.roll(a, -1, axis=1)              # face j: corner j -> j+1
    lo = np.minimum(n1, n2)
    hi = np.maximum(n1, n2)
    key = (lo - 1) * (a.max() + 1) + hi
    flat = key.reshape(-1)
    order = np.argsort(flat, kind="stable")
    sk = flat[order]
    same = sk[1:] == sk[:-1]
    ielel = np.zeros((nel, 4), dtype=np.int32)
    ielfc = np.zeros((nel, 4), dtype=np.int32)
    p = np.nonzero(same)[0]
    fa = order[p]
    fb = order[p + 1]
    ea, ja = fa // 4, fa % 4
    eb, jb = fb // 4, fb % 4
    ielel[ea, ja] = eb + 1
    ielel[eb, jb] = ea + 1
    ielfc[ea, ja] = jb + 1
    ielfc[eb, jb] = ja + 1
    # corrconn: boundary faces point at themselves, side = opposite face
    for j1 in range(2):
        j2 = j1 + 2
        m = ielel[:, j1] == 0
        ielel[m, j1] = np.nonzero(m)[0] + 1
        ielfc[m, j1] = j2 + 1
        m = ielel[:, j2] == 0
        ielel[m, j2] = np.nonzero(m)[0] + 1
        ielfc[m, j2] = j1 + 1
    return ielel, ielfc


def nodetype(ielnd, indtype):
    """init_kn_nodetype (init_kn.f90:78-106): corner nodes between a SLIPX
    and a SLIPY edge become -3.  In place."""
    nnd = indtype.size
    neg = (indtype[ielnd - 1] < 0).sum(axis=1)
    for iel in np.nonzero(neg == 3)[0]:
        nodes = ielnd[iel]
        if np.count_nonzero(indtype[nodes - 1] < 0) != 3:
            continue
        ii = 0
        while ii < 4 and not indtype[nodes[ii] - 1] > 0:
            ii += 1
        ii = (ii + 2) % 4
        jj = nodes[ii]
        if jj <= nnd:
            j1 = nodes[(ii + 1) % 4]
            j2 = nodes[(ii + 3) % 4]
            t1, t2 = indtype[j1 - 1], indtype[j2 - 1]
            if (t1 == -2 and t2 == -1) or (t2 == -2 and t1 == -1):
                indtype[jj - 1] = -3
    return indtype
