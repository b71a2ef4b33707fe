"""A BookLeaf problem on the host: sizes, config and every dataAPI field.

``Problem.from_deck`` runs the reference's set-up sequence (control file,
mesh, connectivity, node types, initial conditions, masses, EoS; see
deck.py, mesh.py, ic.py) and stores each field in a numpy array laid out
as the reference stores it: element fields (nel), corner/face fields as
Fortran (NCORN,nel) blocks -- numpy shape (nel,4), C order -- and node
fields (nnd).  Integer connectivity is 1-based.
"""
import copy

import numpy as np

from .. import abi
from . import deck as deckmod
from . import ic as icmod
from . import mesh as meshmod


class Problem:
    def __init__(self, sizes, config, fields, timestep, name=""):
        self.sizes = sizes
        self.config = config
        self.fields = fields           # {dataAPI id: ndarray}
        self.timestep = timestep
        self.name = name

    # ------------------------------------------------------------------
    @classmethod
    def from_deck(cls, path_or_text, name="", material_fraction=None):
        """The problem a control file describes.  ``material_fraction``, if
        given, replaces the deck's material shapes: a function of the
        elements' corner coordinates (cnx, cny; arrays of shape (nel, 4))
        returning, per element, the volume fraction of material 2 (material
        1 fills the rest; cells strictly between 0 and 1 become mixed cells
        of the two), as a harness can compute exact sub-cell area fractions
        of an interface that the reference's shapes cannot describe."""
        groups = deckmod.read_deck(path_or_text)
        nreg, nmat, regions, materials, rmesh, mmesh = icmod.read_indicators(groups)
        cfg = deckmod.build_config(groups, nreg, nmat)
        ndx, ndy, indtype, ielnd, ielreg_m, ielmat_m = meshmod.generate(
            groups.get("mesh"), cfg.zerocut)
        mesh = meshmod.Mesh(ndx, ndy, indtype, ielnd, ielreg_m, ielmat_m)
        st = icmod.apply(groups, mesh, cfg, nreg, nmat, regions, materials, rmesh, mmesh,
                         material_fraction=material_fraction)
        nel, nnd, ncp, nmx = mesh.nel, mesh.nnd, st["ncp"], st["nmx"]
        s = abi.Sizes()
        s.nel = s.nel1 = s.nel2 = nel
        s.nnd = s.nnd1 = s.nnd2 = nnd
        s.nsz = max(nel, nnd)
        s.nmat, s.nreg, s.ncp, s.nmx = nmat, nreg, ncp, nmx
        s.mcp, s.mmx = ncp, nmx
        f = {}
        d = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        i = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f[abi.ELDENSITY] = d(st["eldensity"])
        f[abi.ELENERGY] = d(st["elenergy"])
        f[abi.ELPRESSURE] = d(st["elpressure"])
        f[abi.ELCS2] = d(st["elcs2"])
        f[abi.ELVOLUME] = d(st["elvolume"])
        for nm, fid in (("a1", abi.A1), ("a2", abi.A2), ("a3", abi.A3), ("b1", abi.B1),
                        ("b2", abi.B2), ("b3", abi.B3)):
            f[fid] = d(st[nm])
        f[abi.CNWT] = d(st["cnwt"])
        f[abi.CNX] = d(st["cnx"])
        f[abi.CNY] = d(st["cny"])
        f[abi.CNVISCX] = np.zeros((nel, 4))
        f[abi.CNVISCY] = np.zeros((nel, 4))
        f[abi.ELVISC] = np.zeros(nel)
        f[abi.ELMASS] = d(st["elmass"])
        f[abi.CNMASS] = d(st["cnmass"])
        f[abi.NDX] = d(mesh.ndx)
        f[abi.NDY] = d(mesh.ndy)
        f[abi.NDU] = d(st["ndu"])
        f[abi.NDV] = d(st["ndv"])
        f[abi.INDTYPE] = i(mesh.indtype)
        f[abi.IELSORT1] = np.arange(1, nel + 1, dtype=np.int32)
        f[abi.IELND] = i(mesh.ielnd)
        f[abi.IELEL] = i(mesh.ielel)
        f[abi.IELFC] = i(mesh.ielfc)
        f[abi.IELMAT] = i(st["ielmat"])
        f[abi.IELREG] = i(st["ielreg"])
        if cfg.ale_zexist:
            f[abi.IELSORT2] = np.arange(1, nel + 1, dtype=np.int32)
        if cfg.zsp:
            f[abi.SPMASS] = d(st["spmass"])
        if ncp > 0:
            f[abi.CPDENSITY] = d(st["cpdensity"])
            f[abi.CPENERGY] = d(st["cpenergy"])
            f[abi.CPPRESSURE] = d(st["cppressure"])
            f[abi.CPCS2] = d(st["cpcs2"])
            f[abi.CPVOLUME] = d(st["cpvolume"])
            f[abi.FRVOLUME] = d(st["frvolume"])
            f[abi.CPMASS] = d(st["cpmass"])
            f[abi.FRMASS] = d(st["frmass"])
            f[abi.CPVISCX] = np.zeros((ncp, 4))
            f[abi.CPVISCY] = np.zeros((ncp, 4))
            f[abi.CPVISC] = np.zeros(ncp)
            f[abi.CPA1] = d(st["cpa1"])
            f[abi.CPA3] = d(st["cpa3"])
            f[abi.CPB1] = d(st["cpb1"])
            f[abi.CPB3] = d(st["cpb3"])
            f[abi.ICPMAT] = i(st["icpmat"])
            f[abi.IMXEL] = i(st["imxel"])
            f[abi.IMXFCP] = i(st["imxfcp"])
            f[abi.IMXNCP] = i(st["imxncp"])
        ts = abi.Timestep()
        ts.time = cfg.time_start          # setup_timestep_rationalise
        ts.dt = cfg.dt_initial
        ts.nstep = 0
        ts.idtel = -1
        ts.imdt = -1
        return cls(s, cfg, f, ts, name)

    # ------------------------------------------------------------------
    def copy(self):
        s = abi.Sizes()
        ct_copy(self.sizes, s)
        c = abi.Config()
        ct_copy(self.config, c)
        return Problem(s, c, {k: v.copy() for k, v in self.fields.items()},
                       self.timestep.copy(), self.name)

    def pointer_table(self):
        return abi.pointer_table(self.fields)

    def __getitem__(self, name):
        return self.fields[abi.IDS[name.upper()]]

    @property
    def nel(self):
        return self.sizes.nel

    @property
    def nnd(self):
        return self.sizes.nnd

    # conservation diagnostics ----------------------------------------------
    def totals(self):
        """Total mass, internal and kinetic energy (hydro_kn_print sums)."""
        f = self.fields
        m = f[abi.ELMASS]
        e = f[abi.ELENERGY]
        u = f[abi.NDU]
        v = f[abi.NDV]
        cnm = f[abi.CNMASS]
        nd = f[abi.IELND] - 1
        ke = 0.5 * np.sum(cnm * (u[nd] ** 2 + v[nd] ** 2))
        return dict(mass=float(np.sum(m)), ie=float(np.sum(m * e)), ke=float(ke))


def ct_copy(src, dst):
    import ctypes as ct
    ct.memmove(ct.addressof(dst), ct.addressof(src), ct.sizeof(src))
