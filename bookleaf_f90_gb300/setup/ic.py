"""Initial conditions and initial state (host side, before the hot path).

Restates the reference's set-up in the order inf_init runs it
(src/infrastructure/init/inf_init.F90:53-103):

  setup_indicator_types / setup_shapes_type / setup_IC_type
                             setup_IC.f90:813-1419 (INDICATORS, SHAPES,
                                                    INITIAL_CONDITIONS)
  setup_regions / setup_materials / setup_flag*
                             setup_IC.f90:268-593, region_shape/material_shape
                             1553-1636, intersect/subdivide 1660-1730
  mix list + flatten         mix_dr_list.f90:46-205 (components of one mixed
                             cell are contiguous, mixed cells in cell order)
  setup_state                setup_IC.f90:321-431 (geometry, thermodynamics,
                             kinematics, boundary conditions)
  init_dr_state              init_dr_utils.f90:95-132 (masses, EoS)
  hydro_dr_init              hydro_dr_init.f90:38-59 (zero viscosity, spmass)

The arithmetic of every formula (geometry, EoS, masses) is evaluated in the
reference's order with IEEE double operations, so the state handed to the
hot path is the state the reference would hand to it.
"""
import numpy as np

from .deck import DeckError, LN, Namelist

MESH_T, BACKGROUND, CELL, SHAPES, REGION, MATERIAL = "MESH", "BACKGROUND", "CELL", "SHAPE", "REGION", "MATERIAL"
MAXIT = 10


def _upper(v):
    return str(v).strip().upper()


def read_indicators(groups):
    """setup_indicator_types (setup_IC.f90:813-1122): ordered indicator lists
    (background first, then cell/mesh/region/material, then shapes)."""
    ind = groups.get("indicators", Namelist())
    rtype = [_upper(v) for v in ind.get_array("region_type", (LN,), "UNKNOWN")]
    rval = [int(v) for v in ind.get_array("region_value", (LN,), -1)]
    mtype = [_upper(v) for v in ind.get_array("material_type", (LN,), "UNKNOWN")]
    mval = [int(v) for v in ind.get_array("material_value", (LN,), -1)]
    nreg = sum(1 for t in rtype if t != "UNKNOWN")
    nmat = sum(1 for t in mtype if t != "UNKNOWN")
    if nreg < 1:
        raise DeckError("ERROR: No regions defined")
    if nmat < 1:
        raise DeckError("ERROR: No materials defined")
    rtype, rval, mtype, mval = rtype[:nreg], rval[:nreg], mtype[:nmat], mval[:nmat]
    if MESH_T in rtype and not all(t == MESH_T for t in rtype):
        raise DeckError("ERROR: Cannot mix region type MESH with other region types")
    if MESH_T in mtype and not all(t == MESH_T for t in mtype):
        raise DeckError("ERROR: Cannot mix material type MESH with other material types")

    def order(types, vals, third):
        out = [(BACKGROUND, vals[i], i + 1) for i, t in enumerate(types) if t == BACKGROUND]
        out += [(t, vals[i], i + 1) for i, t in enumerate(types) if t in (CELL, MESH_T, third)]
        out += [(t, vals[i], i + 1) for i, t in enumerate(types) if t == SHAPES]
        for t in types:
            if t not in (BACKGROUND, CELL, MESH_T, third, SHAPES):
                raise DeckError("ERROR: unrecognised value of %s_type" %
                                ("region" if third == MATERIAL else "material"))
        return out

    regions = order(rtype, rval, MATERIAL)
    materials = order(mtype, mval, REGION)
    return nreg, nmat, regions, materials, all(t == MESH_T for t in rtype), all(t == MESH_T for t in mtype)


def read_shapes(groups):
    """setup_shapes_type (setup_IC.f90:1124-1208)."""
    sh = groups.get("shapes", Namelist())
    stype = [_upper(v) for v in sh.get_array("shape_type", (LN,), "UNKNOWN")]
    sparam = sh.get_array("shape_param", (LN, 5), 0.0)
    forms = []
    for i, t in enumerate(stype):
        if t == "UNKNOWN":
            continue
        p = [float(v) for v in sparam[i, :]]
        if t == "CIRCLE":
            p[3] = 0.0
        elif t != "RECTANGLE":
            raise DeckError("ERROR: unrecognised shape type")
        forms.append((t, p))
    return forms


def read_ic(groups):
    """setup_IC_type (setup_IC.f90:1210-1419)."""
    ic = groups.get("initial_conditions", Namelist())
    ttype = [_upper(v) for v in ic.get_array("thermodynamic_type", (LN,), "UNKNOWN")]
    tval = ic.get_array("thermodynamic_value", (LN,), -1)
    tscale = [_upper(v) for v in ic.get_array("thermodynamic_energy_scale", (LN,), "UNKNOWN")]
    dens = ic.get_array("density", (LN,), -1.0)
    ener = ic.get_array("energy", (LN,), -1.0)
    thermo = []
    for i, t in enumerate(ttype):
        if t == "UNKNOWN":
            continue
        if t not in (REGION, MATERIAL):
            raise DeckError("ERROR: unrecognised thermodynamic type")
        if float(dens[i]) <= 0.0:
            raise DeckError("ERROR: density <= 0")
        if float(ener[i]) < 0.0:
            raise DeckError("ERROR: energy < 0")
        thermo.append(dict(itype=t, param=int(tval[i]), scale=tscale[i],
                           density=float(dens[i]), energy=float(ener[i])))
    if not thermo:
        raise DeckError("ERROR: No initial conditions defined")
    ktype = [_upper(v) for v in ic.get_array("kinematic_type", (LN,), "UNKNOWN")]
    kgeom = [_upper(v) for v in ic.get_array("kinematic_geometry", (LN,), "UNKNOWN")]
    kval = ic.get_array("kinematic_value", (LN,), -1)
    kpar = ic.get_array("kinematic_param", (3, LN), 0.0)
    kin = []
    for i, t in enumerate(ktype):
        if t == "UNKNOWN":
            continue
        if t not in (BACKGROUND, REGION):
            raise DeckError("ERROR: unrecognised kinematic type")
        dat = [float(kpar[j, i]) for j in range(3)]
        if kgeom[i] == "PLANAR":
            dat[2] = 0.0
        elif kgeom[i] != "RADIAL":
            raise DeckError("ERROR: unrecognised kinematic geometry")
        kin.append(dict(itype=t, geom=kgeom[i], param=int(kval[i]), dat=dat))
    return thermo, kin


# ---------------------------------------------------------------- geometry

def centroid(xx, yy):
    """geometry_kn_getcentroid (geometry_kn_centroid.f90:29-55) for rows of
    4 vertices."""
    xx = np.atleast_2d(xx)
    yy = np.atleast_2d(yy)
    n = xx.shape[1]
    cx = np.zeros(xx.shape[0])
    cy = np.zeros(xx.shape[0])
    rvol = np.zeros(xx.shape[0])
    for i1 in range(n):
        i2 = (i1 + 1) % n
        rr = xx[:, i1] * yy[:, i2] - xx[:, i2] * yy[:, i1]
        rvol = rvol + rr
        cx = cx + rr * (xx[:, i1] + xx[:, i2])
        cy = cy + rr * (yy[:, i1] + yy[:, i2])
    rvol = 0.5 * rvol
    with np.errstate(divide="ignore", invalid="ignore"):
        cx = np.where(rvol > 0.0, cx / (6.0 * rvol), 0.0)
        cy = np.where(rvol > 0.0, cy / (6.0 * rvol), 0.0)
    return cx, cy


def _inside(form, px, py):
    t, p = form
    if t == "RECTANGLE":
        return (px > p[0]) & (py > p[1]) & (px < p[2]) & (py < p[3])
    return np.sqrt((px - p[0]) ** 2 + (py - p[1]) ** 2) <= p[2]


def _intersect(form, xx, yy):
    z = _inside(form, np.asarray(xx), np.asarray(yy))
    if np.all(z):
        return 1.0
    if np.any(z):
        return 0.5
    return 0.0


def _subdivide(nit, form, xx, yy):
    """subdivide (setup_IC.f90:1682-1730)."""
    nit_local = nit + 1
    cx, cy = centroid(np.array([xx]), np.array([yy]))
    cx, cy = float(cx[0]), float(cy[0])
    if nit_local > MAXIT:
        return 1.0 if bool(_inside(form, np.array(cx), np.array(cy))) else 0.0
    vf = 0.0
    for ii in range(4):
        jj = (ii + 1) % 4
        kk = (ii + 3) % 4
        xl = [xx[ii], xx[jj], cx, xx[kk]]
        yl = [yy[ii], yy[jj], cy, yy[kk]]
        v = _intersect(form, xl, yl)
        if 0.25 < v < 0.75:
            v = _subdivide(nit_local, form, xl, yl)
        vf = vf + v
    return 0.25 * vf


def getiso(cnx, cny):
    """geometry_kn_getiso + getvolume (geometry_kn_volume.f90:30-79);
    cnx/cny are (nel,4).  Returns a1,a2,a3,b1,b2,b3,cnwt(nel,4),volume."""
    x1, x2, x3, x4 = (cnx[:, j] for j in range(4))
    y1, y2, y3, y4 = (cny[:, j] for j in range(4))
    a1 = 0.25 * (((-x1) + x2) + x3 - x4)
    a2 = 0.25 * (((x1 - x2) + x3) - x4)
    a3 = 0.25 * (((-x1) - x2) + x3 + x4)
    b1 = 0.25 * (((-y1) + y2) + y3 - y4)
    b2 = 0.25 * (((y1 - y2) + y3) - y4)
    b3 = 0.25 * (((-y1) - y2) + y3 + y4)
    o9 = 1.0 / 9.0
    cnwt = np.empty_like(cnx)
    cnwt[:, 0] = o9 * ((3.0 * b3 - b2) * (3.0 * a1 - a2) - (3.0 * a3 - a2) * (3.0 * b1 - b2))
    cnwt[:, 1] = o9 * ((3.0 * b3 + b2) * (3.0 * a1 - a2) - (3.0 * a3 + a2) * (3.0 * b1 - b2))
    cnwt[:, 2] = o9 * ((3.0 * b3 + b2) * (3.0 * a1 + a2) - (3.0 * a3 + a2) * (3.0 * b1 + b2))
    cnwt[:, 3] = o9 * ((3.0 * b3 - b2) * (3.0 * a1 + a2) - (3.0 * a3 - a2) * (3.0 * b1 + b2))
    vol = 4.0 * (a1 * b3 - a3 * b1)
    return a1, a2, a3, b1, b2, b3, cnwt, vol


# ---------------------------------------------------------------- EoS

def eos(cfg, imat, rho, e):
    """eos_kn_getpressure / eos_kn_getcs2 (eos_kn_forms.f90:28-106)."""
    imat = np.maximum(imat, 0)
    p = np.empty_like(rho)
    c2 = np.empty_like(rho)
    for m in np.unique(imat):
        sel = imat == m
        t = cfg.eos_type[m]
        P = [cfg.eos_param[m][k] for k in range(6)]
        r, en = rho[sel], e[sel]
        if t == 0:
            pp = np.full(r.shape, P[0])
            cc = np.full(r.shape, cfg.ccut)
        elif t == 1:
            pp = en * r * (P[0] - 1.0)
            cc = P[0] * (P[0] - 1.0) * en
        elif t == 2:
            t1 = r / P[2]
            pp = P[0] * (t1 ** P[1] - 1.0)
            pp = np.where(P[3] > pp, P[3], pp)
            cc = (P[0] * P[1]) / P[2] * t1 ** (P[1] - 1.0)
        elif t == 3:
            t1 = P[3] * P[5] / r
            t2 = P[4] * P[5] / r
            pp = P[0] * r * en + (1.0 - P[0] / t1) * P[1] * np.exp(-t1) + (1.0 - P[0] / t2) * P[2] * np.exp(-t2)
            pp = np.where(np.abs(pp) < cfg.pcut, 0.0, pp)
            q1 = P[5] / r
            s3 = P[3] * q1
            t4 = (P[0] / P[3] + P[0] * q1 - s3 * q1) * P[1] * np.exp(-s3)
            s3 = P[4] * q1
            t5 = (P[0] / P[4] + P[0] * q1 - s3 * q1) * P[2] * np.exp(-s3)
            cc = P[0] * pp / r + P[0] * en - t4 - t5
        else:
            pp = np.full(r.shape, -1.0)
            cc = np.full(r.shape, cfg.ccut)
        pp = np.where(np.abs(pp) < cfg.pcut, 0.0, pp)
        cc = np.where(cfg.ccut > cc, cfg.ccut, cc)
        p[sel] = pp
        c2[sel] = cc
    return p, c2


# ---------------------------------------------------------------- IC driver

def apply(groups, mesh, cfg, nreg, nmat, regions, materials, rmesh, mmesh,
          material_fraction=None):
    """Return the dict of initial fields for the mesh (setup_IC + init).
    ``material_fraction`` (see Problem.from_deck) overrides the material
    shapes with per-cell volume fractions of material 2."""
    forms = read_shapes(groups)
    thermo, kin = read_ic(groups)
    nel, nnd = mesh.nel, mesh.nnd
    ielnd = mesh.ielnd
    cnx = mesh.ndx[ielnd - 1]
    cny = mesh.ndy[ielnd - 1]
    # setup_regions (setup_IC.f90:268-290)
    ielreg = mesh.ielreg.copy() if rmesh else np.zeros(nel, np.int32)
    _flag(regions, ielreg, mesh.ielmat, cnx, cny, forms, None)
    if np.any(ielreg == 0):
        raise DeckError("ERROR: region not fully populated")
    # setup_materials (setup_IC.f90:292-319)
    ielmat = mesh.ielmat.copy() if mmesh else np.zeros(nel, np.int32)
    mix = {}                      # iel (1-based) -> list of (material, fraction)
    _flag(materials, ielmat, ielreg, cnx, cny, forms, mix)
    if material_fraction is not None:
        if nmat < 2:
            raise DeckError("ERROR: a material fraction needs two materials")
        vf = np.asarray(material_fraction(cnx, cny), dtype=np.float64)
        mix = {}
        ielmat = np.where(vf >= 1.0, 2, 1).astype(np.int32)
        for iel in np.nonzero((vf > 0.0) & (vf < 1.0))[0]:
            mix[int(iel) + 1] = [(1, 1.0 - float(vf[iel])), (2, float(vf[iel]))]
    if np.any(ielmat == 0):
        raise DeckError("ERROR: material not fully populated")
    # flatten: mixed cells in cell order, their components contiguous
    mixed = sorted(mix)
    nmx = len(mixed)
    ncp = sum(len(mix[i]) for i in mixed)
    imxel = np.array(mixed, dtype=np.int32)
    imxncp = np.array([len(mix[i]) for i in mixed], dtype=np.int32)
    imxfcp = (np.concatenate([[1], 1 + np.cumsum(imxncp)[:-1]]).astype(np.int32)
              if nmx else np.zeros(0, np.int32))
    icpmat = np.array([m for i in mixed for (m, f) in mix[i]], dtype=np.int32)
    frvolume = np.array([f for i in mixed for (m, f) in mix[i]], dtype=np.float64)
    for imx, iel in enumerate(mixed):
        ielmat[iel - 1] = -(imx + 1)
    # setup_state: geometry (setup_IC.f90:333)
    a1, a2, a3, b1, b2, b3, cnwt, vol = getiso(cnx, cny)
    if np.any(vol < 0.0):
        raise DeckError("ERROR: negative volume in geometry_dr_getgeometry")
    cp_el = np.repeat(imxel, imxncp) if ncp else np.zeros(0, np.int32)
    cpvolume = (4.0 * (a1[cp_el - 1] * b3[cp_el - 1] - a3[cp_el - 1] * b1[cp_el - 1])) * frvolume
    rho = np.zeros(nel)
    e = np.zeros(nel)
    cprho = np.zeros(ncp)
    cpe = np.zeros(ncp)
    for t in thermo:
        if t["itype"] == REGION:
            _thermo(t, ielreg, vol, rho, e)
        else:
            _thermo(t, ielmat, vol, rho, e)
            if ncp:
                _thermo(t, icpmat, cpvolume, cprho, cpe)
    if ncp and any(t["itype"] == REGION for t in thermo):
        # setup_thermodynamic_rationalise (setup_IC.f90:740-787)
        matset = {t["param"] for t in thermo if t["itype"] == MATERIAL}
        mtypes = {m[2]: m[0] for m in materials}
        for icp in range(ncp):
            m = int(icpmat[icp])
            if m not in matset:
                if mtypes.get(m) in (REGION, BACKGROUND):
                    cprho[icp] = rho[cp_el[icp] - 1]
                    cpe[icp] = e[cp_el[icp] - 1]
                else:
                    raise DeckError("ERROR: failed to rationalise thermodynamic IC due to incorrect material type")
    # kinematics (setup_IC.f90:372-380, 631-811)
    u = np.zeros(nnd)
    v = np.zeros(nnd)
    wt = np.zeros(nnd) if any(k["itype"] == REGION for k in kin) else None
    for k in kin:
        d = k["dat"]
        if k["itype"] == BACKGROUND:
            if k["geom"] == "RADIAL":
                with np.errstate(divide="ignore", invalid="ignore"):
                    rv = 1.0 / np.sqrt((mesh.ndx - d[1]) ** 2 + (mesh.ndy - d[2]) ** 2)
                    u = d[0] * mesh.ndx * rv
                    v = d[0] * mesh.ndy * rv
            else:
                u = np.full(nnd, d[0])
                v = np.full(nnd, d[1])
        else:
            sel = np.nonzero(ielreg == k["param"])[0]
            if k["geom"] == "RADIAL":
                px, py = centroid(cnx[sel], cny[sel])
                rv = 1.0 / np.sqrt((px - d[1]) ** 2 + (py - d[2]) ** 2)
            for iel_i, iel in enumerate(sel):
                for ic in range(4):
                    ind = ielnd[iel, ic] - 1
                    if k["geom"] == "RADIAL":
                        u[ind] = u[ind] + cnwt[iel, ic] * px[iel_i] * rv[iel_i] * d[0]
                        v[ind] = v[ind] + cnwt[iel, ic] * py[iel_i] * rv[iel_i] * d[1]
                    else:
                        u[ind] = u[ind] + cnwt[iel, ic] * d[0]
                        v[ind] = v[ind] + cnwt[iel, ic] * d[1]
                    wt[ind] = wt[ind] + cnwt[iel, ic]
    if wt is not None:
        small = np.abs(wt) < cfg.zerocut
        with np.errstate(divide="ignore", invalid="ignore"):
            rv = 1.0 / wt
        u = np.where(small, 0.0, u * rv)
        v = np.where(small, 0.0, v * rv)
    # utils_dr_bc with accut (utils_kn_bc.f90:28-58)
    _bc(mesh.indtype, u, v, cfg.accut)
    if np.any(rho <= 0.0):
        raise DeckError("ERROR: eldensity not positive")
    if np.any(e < 0.0):
        raise DeckError("ERROR: elenergy negative")
    # init_dr_state: masses (init_kn.f90:32-63) and EoS
    elmass = rho * vol
    cnmass = rho[:, None] * cnwt
    cpmass = cprho * cpvolume
    frmass = cpmass / elmass[cp_el - 1] if ncp else np.zeros(0)
    p, cs2 = eos(cfg, ielmat, rho, e)
    cpp, cpcs2 = eos(cfg, icpmat, cprho, cpe) if ncp else (np.zeros(0), np.zeros(0))
    # hydro_dr_init: spmass (hydro_kn_init.f90:46-77)
    spmass = _spmass(rho, cnx, cny) if cfg.zsp else None
    return dict(
        ielreg=ielreg, ielmat=ielmat, cnx=cnx, cny=cny, a1=a1, a2=a2, a3=a3, b1=b1,
        b2=b2, b3=b3, cnwt=cnwt, elvolume=vol, eldensity=rho, elenergy=e, ndu=u, ndv=v,
        elmass=elmass, cnmass=cnmass, elpressure=p, elcs2=cs2, spmass=spmass,
        nmx=nmx, ncp=ncp, imxel=imxel, imxfcp=imxfcp, imxncp=imxncp, icpmat=icpmat,
        frvolume=frvolume, cpvolume=cpvolume, cpdensity=cprho, cpenergy=cpe,
        cpmass=cpmass, frmass=frmass, cppressure=cpp, cpcs2=cpcs2,
        cpa1=a1[cp_el - 1], cpa3=a3[cp_el - 1], cpb1=b1[cp_el - 1], cpb3=b3[cp_el - 1],
    )


def _flag(indicators, iflag, itest, cnx, cny, forms, mix):
    """setup_flag (setup_IC.f90:433-486) for regions (mix is None) or
    materials (mix collects mixed cells, material_shape)."""
    for itype, param, inumber in indicators:
        if itype == MESH_T:
            break
        if itype == BACKGROUND:
            iflag[:] = inumber
        elif itype == CELL:
            if not 1 <= param <= iflag.size:
                raise DeckError("ERROR: incorrect cell index in setup_flag_cell")
            iflag[param - 1] = inumber
        elif itype in (REGION, MATERIAL):
            iflag[itest == param] = inumber
        elif itype == SHAPES:
            if not 1 <= param <= len(forms):
                raise DeckError("ERROR: failed to find shape")
            form = forms[param - 1]
            if mix is None:
                px, py = centroid(cnx, cny)
                iflag[_inside(form, px, py)] = inumber
            else:
                for ii in range(iflag.size):
                    vf = _intersect(form, cnx[ii], cny[ii])
                    if vf > 0.75:
                        iflag[ii] = inumber
                    elif vf > 0.25:
                        vf = form[1][4] if form[1][4] > 0.0 else _subdivide(0, form, list(cnx[ii]), list(cny[ii]))
                        jj = int(iflag[ii])
                        if jj > 0:
                            mix[ii + 1] = [(jj, 1.0 - vf)]
                            iflag[ii] = -1
                        mix.setdefault(ii + 1, []).append((inumber, vf))
        else:
            raise DeckError("ERROR: unrecognised indicator type")


def _thermo(t, iflag, vol, rho, e):
    """setup_thermodynamic (setup_IC.f90:595-629)."""
    sel = iflag == t["param"]
    rho[sel] = t["density"]
    e[sel] = t["energy"]
    if t["scale"] == "VOLUME":
        e[sel] = e[sel] / vol[sel]
    elif t["scale"] == "MASS":
        e[sel] = e[sel] / (rho[sel] * vol[sel])


def _bc(indtype, u, v, rcut):
    u[(indtype == -1) | (indtype == -3)] = 0.0
    v[(indtype == -2) | (indtype == -3)] = 0.0
    w2 = u * u + v * v
    small = w2 < rcut * rcut
    u[small] = 0.0
    v[small] = 0.0


def _spmass(rho, cnx, cny):
    x3 = 0.25 * (((cnx[:, 0] + cnx[:, 1]) + cnx[:, 2]) + cnx[:, 3])
    y3 = 0.25 * (((cny[:, 0] + cny[:, 1]) + cny[:, 2]) + cny[:, 3])
    sp = np.empty_like(cnx)
    for j1 in range(4):
        x1, y1 = cnx[:, j1], cny[:, j1]
        j2 = (j1 + 1) % 4
        x2 = 0.5 * (x1 + cnx[:, j2])
        y2 = 0.5 * (y1 + cny[:, j2])
        j2 = (j1 + 3) % 4
        x4 = 0.5 * (x1 + cnx[:, j2])
        y4 = 0.5 * (y1 + cny[:, j2])
        w1 = 0.25 * ((((-x1) + x2) + x3) - x4)
        w2 = 0.25 * ((((-x1) - x2) + x3) + x4)
        w3 = 0.25 * ((((-y1) + y2) + y3) - y4)
        w4 = 0.25 * ((((-y1) - y2) + y3) + y4)
        sp[:, j1] = 4.0 * rho * (w1 * w4 - w2 * w3)
    return sp
