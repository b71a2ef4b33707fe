"""Device diagnostics (bl_shortprint, bl_check_sod) against the reference's
formulas evaluated on the host from the synced fields (hydro_kn_print.F90,
hydro_dr_print.f90, check_kn_tests.f90).  Sums may differ in rounding only
(fixed-tree vs serial order); extremes are exact."""
import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, Solver, abi, configs

pytestmark = pytest.mark.gpu


def _calc(nflag, dencut, flag, rho, e, p, vol, m, cnwt, cnu, cnv, acc):
    """hydro_kn_calc_shortprint, serially, into acc (dict of arrays)."""
    for ii in range(flag.size):
        f = int(flag[ii])
        if f <= 0:
            continue
        k = f - 1
        acc["vol"][k] += vol[ii]
        if m[ii] > dencut * vol[ii]:
            acc["mass"][k] += m[ii]
            acc["ie"][k] += e[ii] * m[ii]
            acc["pre"][k] += m[ii] * p[ii]
            acc["pmx"][k] = max(acc["pmx"][k], p[ii])
            acc["pmn"][k] = min(acc["pmn"][k], p[ii])
            acc["dmx"][k] = max(acc["dmx"][k], rho[ii])
            acc["dmn"][k] = min(acc["dmn"][k], rho[ii])
            for ic in range(4):
                acc["ke"][k] += 0.5 * cnwt[ii, ic] * rho[ii] * (cnu[ii, ic] ** 2 + cnv[ii, ic] ** 2)


def _reference_tables(pr):
    f = pr.fields
    nd = f[abi.IELND] - 1
    cnu, cnv = f[abi.NDU][nd], f[abi.NDV][nd]
    dencut = pr.config.dencut
    out = []
    for table, nflag, flag in ((0, pr.sizes.nreg, f[abi.IELREG]), (1, pr.sizes.nmat, f[abi.IELMAT])):
        acc = {k: np.zeros(nflag) for k in ("vol", "mass", "ie", "ke", "pre")}
        acc.update(pmn=np.full(nflag, np.finfo(float).max), pmx=np.full(nflag, -np.finfo(float).max),
                   dmn=np.full(nflag, np.finfo(float).max), dmx=np.full(nflag, -np.finfo(float).max))
        _calc(nflag, dencut, flag, f[abi.ELDENSITY], f[abi.ELENERGY], f[abi.ELPRESSURE],
              f[abi.ELVOLUME], f[abi.ELMASS], f[abi.CNWT], cnu, cnv, acc)
        if table == 1 and pr.sizes.ncp > 0:
            el = np.repeat(f[abi.IMXEL] - 1, f[abi.IMXNCP])
            _calc(nflag, dencut, f[abi.ICPMAT], f[abi.CPDENSITY], f[abi.CPENERGY],
                  f[abi.CPPRESSURE], f[abi.CPVOLUME], f[abi.CPMASS], f[abi.CNWT][el], cnu[el],
                  cnv[el], acc)
        rows = []
        for k in range(nflag):
            dens = acc["mass"][k] / acc["vol"][k] if acc["vol"][k] > 0 else 0.0
            pres = (acc["pre"][k] / acc["mass"][k] if acc["mass"][k] > dencut * acc["vol"][k]
                    else acc["pre"][k])
            rows.append(dict(vol=acc["vol"][k], mass=acc["mass"][k], ie=acc["ie"][k], ke=acc["ke"][k],
                             pressure=pres, pmn=acc["pmn"][k], pmx=acc["pmx"][k], density=dens,
                             dmn=acc["dmn"][k], dmx=acc["dmx"][k]))
        out.append(rows)
    return out


@pytest.mark.parametrize("deck", [configs.sod_multimaterial(40, 10), configs.sedov(24, kappa=0.01)])
def test_shortprint_matches_reference_formulas(deck):
    p = Problem.from_deck(deck)
    s = Solver(p, fp_mode=abi.FP_EXACT)
    for _ in range(12):
        assert s.step() == 0, s.error.message
    reg, mat = s.shortprint(False), s.shortprint(True)
    s.sync_to_host(0)
    ref_reg, ref_mat = _reference_tables(p)
    for got, ref in ((reg, ref_reg), (mat, ref_mat)):
        assert len(got) == len(ref)
        for g, r in zip(got, ref):
            for k in ("pmn", "pmx", "dmn", "dmx"):
                assert g[k] == r[k], (k, g[k], r[k])
            for k in ("vol", "mass", "ie", "ke", "pressure", "density"):
                assert abs(g[k] - r[k]) <= 1e-12 * max(abs(r[k]), 1e-300), (k, g[k], r[k])


def test_check_sod_matches_restatement():
    from oracle.oracle import sod_l1
    p = Problem.from_deck(configs.sod_reference(100, 5, time_end=5.0))
    s = Solver(p, fp_mode=abi.FP_EXACT)
    ierr, _ = s.run(history=False)
    assert ierr == 0
    d, e = s.check_sod()
    s.sync_to_host(0)
    rd, re_ = sod_l1(p, p.timestep.time)
    assert abs(d - rd) <= 1e-12 * rd and abs(e - re_) <= 1e-12 * re_, ((d, e), (rd, re_))
