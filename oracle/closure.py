"""CPU restatement of one step of the learned mixed-cell closure
(k_mix_closure in bookleaf_f90_gb300/csrc/hydro_kernels.cuh), for the GPU
parity test of that kernel.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker.  Never used by
the product.

The closure has no counterpart in the reference: it replaces, for
two-material cells, the component update of the reference's Lagrangian step
(hydro_kn_getenergy.f90 / density_dr_getdensity.f90 applied to components,
each material keeping its volume fraction), which the oracle's own lagstep
performs.  ``apply`` takes the state that plain step left (the plain
closure's components after the step), the components' state before it, and
the network, and makes the closure's changes in place:

  features (t^n): fr1, rho1, rho2, p1, p2, cs2_1, cs2_2, dV/V^n,
      dt sqrt(max cs2 / V^n), (p1 - p2) / (|p1| + |p2|), standardised in
      FP32 as (f - norm[k]) * norm[10 + k];
  network: oracle/mlp.py's forward with the operands rounded to BF16;
  exchange: x = norm[20] (y1 - y2) / 2 into material 1, clamped to [0, x_eq]
      with x_eq = (p1' - p2') V^{n+1} / (V^n (rho1' c1'^2 / fr1 + rho2' c2'^2 / fr2))
      from the plain step's state (');
  accepted when the outputs are finite, |y1 + y2| <= norm[21], x lies no
      farther than |x_eq| outside [0, x_eq], and both volumes stay positive;
  accepted cells: V_m = V_m' + x_m V^n, e_m = e_m' - p_bar x_m V^n / M_m (mode 1
      only; p_bar = fr1 p1 + fr2 p2 at t^n), then density, EoS and fraction.
"""
import numpy as np

from . import mlp


def apply(f, before, dt, params, norm, mode, eos, zerocut=0.0):
    """f: the problem's field dict after the plain step (component arrays
    updated in place); before: dict of the components' t^n arrays (frvol,
    cprho, cpp, cpcs2) and the mixed cells' t^n volume 'vol0' (per mixed
    cell); eos(imat, rho, e) -> (p, cs2).  Returns the accepted mask."""
    from bookleaf_f90_gb300 import abi
    nmx = len(before["vol0"])
    el = f[abi.IMXEL][:nmx] - 1
    c0 = f[abi.IMXFCP][:nmx] - 1
    V0 = before["vol0"]
    V1 = f[abi.ELVOLUME][el]
    fr = np.stack([before["frvol"][c0], before["frvol"][c0 + 1]], axis=1)
    rho = np.stack([before["cprho"][c0], before["cprho"][c0 + 1]], axis=1)
    p = np.stack([before["cpp"][c0], before["cpp"][c0 + 1]], axis=1)
    q = np.stack([before["cpcs2"][c0], before["cpcs2"][c0 + 1]], axis=1)
    raw = np.stack([fr[:, 0], rho[:, 0], rho[:, 1], p[:, 0], p[:, 1], q[:, 0], q[:, 1],
                    (V1 - V0) / V0, dt * np.sqrt(np.maximum(q[:, 0], q[:, 1]) / V0),
                    (p[:, 0] - p[:, 1]) / (np.abs(p[:, 0]) + np.abs(p[:, 1]) + 1e-300)], axis=1)
    n32 = np.asarray(norm, dtype=np.float32)
    x = (raw.astype(np.float32) - n32[:10]) * n32[10:20]
    y, _ = mlp.forward(params, x, bf=True)
    y = y.astype(np.float32)
    # the plain step's state of both materials
    cp = lambda fid: np.stack([f[fid][c0], f[fid][c0 + 1]], axis=1)
    pe, pv, pr, pp, pc = (cp(abi.CPENERGY), cp(abi.CPVOLUME), cp(abi.CPDENSITY),
                          cp(abi.CPPRESSURE), cp(abi.CPCS2))
    xeq = (pp[:, 0] - pp[:, 1]) * V1 / (V0 * (pr[:, 0] * pc[:, 0] / fr[:, 0] +
                                              pr[:, 1] * pc[:, 1] / fr[:, 1]))
    lo, hi, m = np.minimum(0.0, xeq), np.maximum(0.0, xeq), np.abs(xeq)
    xp = 0.5 * float(n32[20]) * (y[:, 0].astype(np.float64) - y[:, 1].astype(np.float64))
    xm = np.minimum(np.maximum(xp, lo), hi)
    ok = (np.all(np.isfinite(y), axis=1) & np.isfinite(xeq) &
          (np.abs(y[:, 0] + y[:, 1]) <= n32[21]) & (xp >= lo - m) & (xp <= hi + m) &
          (V1 * fr[:, 0] + xm * V0 > 0.0) & (V1 * fr[:, 1] - xm * V0 > 0.0))
    pbar = fr[:, 0] * p[:, 0] + fr[:, 1] * p[:, 1]
    for k, xk in ((0, xm), (1, -xm)):
        icp = (c0 + k)[ok]
        cpm = f[abi.CPMASS][icp]
        cpv = pv[ok, k] + xk[ok] * V0[ok]
        cpe = pe[ok, k]
        if mode == 1:
            cpe = cpe - pbar[ok] * (xk[ok] * V0[ok]) / np.maximum(cpm, zerocut)
        cpr = cpm / cpv
        ppn, pcn = eos(f[abi.ICPMAT][icp], cpr, cpe)
        f[abi.CPVOLUME][icp] = cpv
        f[abi.CPENERGY][icp] = cpe
        f[abi.CPDENSITY][icp] = cpr
        f[abi.CPPRESSURE][icp] = ppn
        f[abi.CPCS2][icp] = pcn
        f[abi.FRVOLUME][icp] = cpv / V1[ok]
    return ok
