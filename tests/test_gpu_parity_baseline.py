"""Parity at the benchmark configurations' own sizes, and on the
reference's own control files, through the C-ABI.

Each case runs the CPU restatement once from t = 0 and keeps its state at
a few checkpoint steps and its per-step (nstep, time, dt, idtel, sdt)
record; the device time loop (bl_run, the path the benchmark times) then
runs the same steps in both floating-point modes:

- exact mode (no FMA contraction): every step's timestep record equal, and
  every state field equal bit for bit at every checkpoint;
- fast mode: at the last checkpoint, total mass and total energy within
  1e-12 relative, and density, specific energy and the velocity field
  within 1e-9 L1 relative (sum |gpu - cpu| / sum |cpu|).

Configurations: Sod 400x40 to t = 0.2 (checkpoints every 50 steps),
Sedov 512x512 with the benchmark's hourglass and sub-zonal settings for
100 steps, Sedov 128x128 with them to t = 1, Noh 2048x2048 Lagrangian and
Eulerian for 5 steps, Noh Lagrangian on the reference's own polar mesh
(150x60, the family of input/noh_small) to t = 0.6, and the two-material
Sod at 2000x200 with its mixed cells for 200 steps.
"""
import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, Solver, abi, configs
from helpers import compare, state_ids

import golden

pytestmark = pytest.mark.gpu

L1_TOL = 1e-9
SUM_TOL = 1e-12


def _record(ts):
    return (ts.nstep, ts.time, ts.dt, ts.idtel, ts.sdt.decode().strip())


def _oracle_run(base, nsteps, every):
    """The restatement from t = 0: (records, {step: (timestep, fields)}).
    nsteps None runs to time_end.  Checkpoints at multiples of `every` and
    at the last step."""
    from oracle.oracle import Oracle
    p = base.copy()
    o = Oracle(p)
    ts = p.timestep
    recs, cps = [], {}
    n = 0
    while True:
        ierr = o.step(ts)
        assert ierr == 0, o.err.message
        n += 1
        recs.append(_record(ts))
        last = (n == nsteps) if nsteps else (ts.time >= p.config.time_end)
        if last or (every and n % every == 0):
            cps[n] = (ts.copy(), {fid: p.fields[fid].copy() for fid in state_ids(p)})
        if last:
            return recs, cps


_CACHE = {}


def _oracle(name, deck, nsteps, every):
    if name not in _CACHE:
        _CACHE.clear()   # keep one case's checkpoints in host memory at a time
        base = deck if isinstance(deck, Problem) else Problem.from_deck(deck)
        _CACHE[name] = (base, _oracle_run(base, nsteps, every))
    return _CACHE[name]


def _as_problem(base, ts, fields):
    q = base.copy()
    q.timestep = ts.copy()
    for fid, a in fields.items():
        np.copyto(q.fields[fid], a)
    return q


def _check_fast(pg, pc):
    tg, tc = pg.totals(), pc.totals()
    assert abs(tg["mass"] - tc["mass"]) <= SUM_TOL * abs(tc["mass"])
    eg, ec = tg["ie"] + tg["ke"], tc["ie"] + tc["ke"]
    assert abs(eg - ec) <= SUM_TOL * abs(ec), (eg, ec)
    for fid in (abi.ELDENSITY, abi.ELENERGY):
        a, b = pg.fields[fid], pc.fields[fid]
        l1 = np.sum(np.abs(a - b)) / max(np.sum(np.abs(b)), 1e-300)
        assert l1 <= L1_TOL, (abi.NAMES[fid], l1)
    du = (np.abs(pg.fields[abi.NDU] - pc.fields[abi.NDU])
          + np.abs(pg.fields[abi.NDV] - pc.fields[abi.NDV]))
    un = np.abs(pc.fields[abi.NDU]) + np.abs(pc.fields[abi.NDV])
    assert np.sum(du) <= L1_TOL * np.sum(un), np.sum(du) / np.sum(un)


def _device_run(base, recs, cps, mode):
    """Device loop over the oracle's steps in chunks ending at each
    checkpoint; compares as the module docstring says."""
    pg = base.copy()
    s = Solver(pg, fp_mode=mode)
    ts = pg.timestep
    done = 0
    hist = []
    try:
        for step in sorted(cps):
            ierr, h = s.run(max_steps=step - done, ts=ts)
            assert ierr == 0, s.error.message
            hist += h
            done = step
            assert ts.nstep == step
            if mode == abi.FP_EXACT:
                s.sync_to_host(0)
                pc = _as_problem(base, *cps[step])
                bad = compare(pg, pc, exact=True, where="step %d" % step)
                assert not bad, "\n".join(bad[:10])
        if mode == abi.FP_EXACT:
            got = [(r[0], r[1], r[2], r[3], r[4].strip()) for r in hist]
            assert got == recs[:len(got)] and len(got) == len(recs)
        else:
            s.sync_to_host(0)
            last = max(cps)
            _check_fast(pg, _as_problem(base, *cps[last]))
            # the run's length matches within a step or two at the end time
            assert abs(len(hist) - len(recs)) <= 2
    finally:
        s.close()


BASELINE = {
    # name: (deck, steps (None: to time_end), checkpoint every)
    "sod_400x40_t0.2": (lambda: configs.sod(400, 40, time_end=0.2), None, 50),
    "sedov_512_bench_100steps": (lambda: configs.sedov(512, kappa=0.01, pmerit=0.1), 100, 50),
    "sedov_128_bench_t1": (lambda: configs.sedov(128, kappa=0.01, pmerit=0.1), None, 0),
    "noh_2048_lagrangian_5steps": (lambda: configs.noh(2048), 5, 0),
    "noh_2048_eulerian_5steps": (lambda: configs.noh(2048, eulerian=True), 5, 0),
    # the reference's own polar Noh mesh (input/noh_small's family), to t = 0.6
    "noh_polar_150x60_t0.6": (lambda: configs.noh_polar(150, 60), None, 2000),
    # the two-material Sod at its stated size with mixed cells: the planar
    # interface tilted by 0.2 (right state rho = p = 0.5) the closure
    # benchmark measures, cells cut by it made mixed with their exact area
    # fractions; 200 steps
    "sod2mat_2000x200_tilted_200steps": (lambda: _sod2mat(2000, 200), 200, 100),
}


def _sod2mat(nx, ny):
    deck, frac = configs.sod_interface(nx, ny, time_end=0.2, amplitude=0.0, periods=0,
                                       tilt=0.2, rho_right=0.5, p_right=0.5)
    return Problem.from_deck(deck, material_fraction=frac)


@pytest.mark.parametrize("mode", [abi.FP_EXACT, abi.FP_FAST], ids=["exact", "fast"])
@pytest.mark.parametrize("name", list(BASELINE))
def test_baseline_configuration(name, mode):
    deck, nsteps, every = BASELINE[name]
    base, (recs, cps) = _oracle(name, deck(), nsteps, every)
    if mode == abi.FP_FAST and nsteps is None:
        # to the end time, fast mode may take a step more or fewer: compare
        # at the oracle's last step count instead of the end time
        last = max(cps)
        cps = {last: cps[last]}
    _device_run(base, recs, cps, mode)


# The reference's control files (tests/golden/decks).  The small decks run
# 20 steps with a comparison after every solver call; the 1M-element
# ("medium") decks 8 steps and the 14M-element ("large") ones 2, compared
# after the last call.
def _deck_cases():
    out = []
    for name in golden.deck_names():
        out.append((name, 2 if name.endswith("_large") else 8 if name.endswith("_medium") else 20))
    return out


@pytest.mark.parametrize("name,steps", _deck_cases())
def test_reference_deck_exact(name, steps):
    from helpers import run_pair
    _, _, bad = run_pair(golden.deck_text(name), steps, exact=True, phases=steps == 20)
    assert not bad, "\n".join(bad[:10])
