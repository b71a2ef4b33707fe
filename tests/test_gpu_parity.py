"""Parity of the sm_103a path with the CPU restatement, through the C-ABI.

Exact mode (BL_FP_EXACT, no fused multiply-add) must reproduce the
restatement bit for bit after every solver call.  Fast mode (FMA allowed)
must stay within these tolerances of it: total mass and energy to 1e-12
relative and density, energy and velocity fields within 1e-9 L1 relative.
"""
import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, Solver, abi, configs
from helpers import compare, run_pair

pytestmark = pytest.mark.gpu

HG = configs.sedov(16).replace("cvisc2=0.75\n", "cvisc2=0.75\n kappaall=0.05\n pmeritall=0.3\n")
DTNOT = configs.sod(24, 4).replace(
    "cvisc2=0.75\n", "cvisc2=0.75\n zmidlength(2)=.TRUE.\n zdtnotreg(1)=.TRUE.\n")
TENSOR = configs.sod(24, 4).replace("cvisc2=0.75\n", "cvisc2=0.75\n visc='TENSOR'\n")

CASES = {
    "sod_lag": (configs.sod(40, 6), 25),
    "sod_ref_geometry": (configs.sod_reference(50, 5), 20),
    "sedov_lag": (configs.sedov(24), 25),
    "noh_lag": (configs.noh(24), 20),
    "noh_eul": (configs.noh(24, eulerian=True), 20),
    "sedov_eul": (configs.sedov(20, eulerian=True), 20),
    "sod_eul": (configs.sod(40, 4, eulerian=True), 20),
    "sod_multimaterial": (configs.sod_multimaterial(40, 10), 20),
    "hourglass_subzonal": (HG, 20),
    "dtnotreg_midlength": (DTNOT, 15),
    "tensor_viscosity_off": (TENSOR, 10),
    # the void, Tait and JWL equations of state (eos_kn_forms.f90:28-106),
    # each for material 2 with a column of mixed cells
    "eos_void": (configs.eos_tube("void", 60, 6), 20),
    "eos_tait": (configs.eos_tube("tait", 60, 6), 20),
    "eos_jwl": (configs.eos_tube("jwl", 60, 6), 20),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_exact_per_phase(name):
    deck, n = CASES[name]
    _, _, bad = run_pair(deck, n, exact=True, phases=True)
    assert not bad, "\n".join(bad[:10])


@pytest.mark.parametrize("name", ["sod_lag", "sedov_lag", "noh_eul", "sod_multimaterial",
                                  "hourglass_subzonal", "eos_tait", "eos_jwl"])
def test_fast_within_tolerance(name):
    deck, n = CASES[name]
    pg, pc, bad = run_pair(deck, n, exact=False, phases=False, rtol=1e-9, atol=1e-12)
    tg, tc = pg.totals(), pc.totals()
    assert abs(tg["mass"] - tc["mass"]) <= 1e-12 * abs(tc["mass"])
    et, ec = tg["ie"] + tg["ke"], tc["ie"] + tc["ke"]
    assert abs(et - ec) <= 1e-12 * abs(ec)
    for fid in (abi.ELDENSITY, abi.ELENERGY):
        a, b = pg.fields[fid], pc.fields[fid]
        l1 = np.sum(np.abs(a - b)) / max(np.sum(np.abs(b)), 1e-300)
        assert l1 <= 1e-9, (abi.NAMES[fid], l1)
    # the velocity field as a whole (in Sod the y component is round-off)
    du = np.abs(pg.fields[abi.NDU] - pc.fields[abi.NDU]) + np.abs(pg.fields[abi.NDV] - pc.fields[abi.NDV])
    un = np.abs(pc.fields[abi.NDU]) + np.abs(pc.fields[abi.NDV])
    assert np.sum(du) <= 1e-9 * np.sum(un), np.sum(du) / np.sum(un)


def test_device_loop_matches_per_call():
    """bl_run (device time loop, CUDA graphs) equals the per-call path."""
    base = Problem.from_deck(configs.sedov(24, time_end=0.02))
    pa, pb = base.copy(), base.copy()
    sa = Solver(pa, fp_mode=abi.FP_EXACT)
    steps = 0
    while True:
        assert sa.step() == 0
        steps += 1
        if pa.timestep.time >= pa.config.time_end:
            break
    sa.sync_to_host(0)
    sb = Solver(pb, fp_mode=abi.FP_EXACT)
    ierr, hist = sb.run()
    assert ierr == 0, sb.error.message
    sb.sync_to_host(0)
    assert len(hist) == steps
    assert pb.timestep.nstep == pa.timestep.nstep
    assert pb.timestep.time == pa.timestep.time
    assert not compare(pb, pa, exact=True)


def test_device_loop_history_toggle():
    """Runs with and without a history buffer in turn: each run's records are
    its own steps, and the state matches the per-call path."""
    base = Problem.from_deck(configs.sedov(16, time_end=1.0))
    pa, pb = base.copy(), base.copy()
    sa = Solver(pa, fp_mode=abi.FP_EXACT)
    ierr, h1 = sa.run(max_steps=20)
    assert ierr == 0 and [r[0] for r in h1] == list(range(1, 21))
    ierr, h2 = sa.run(max_steps=20, history=False)
    assert ierr == 0 and h2 == []
    ierr, h3 = sa.run(max_steps=20)
    assert ierr == 0 and [r[0] for r in h3] == list(range(41, 61))
    sb = Solver(pb, fp_mode=abi.FP_EXACT)
    times = []
    for _ in range(60):
        assert sb.step() == 0
        times.append(pb.timestep.time)
    assert [r[1] for r in h1] == times[:20]
    assert [r[1] for r in h3] == times[40:]
    sa.sync_to_host(0)
    sb.sync_to_host(0)
    assert not compare(pa, pb, exact=True)


def test_restart_from_host_state():
    """bl_sync_to_device replaces the whole device state: a context that ran
    a few steps and is then given its initial fields again runs exactly as a
    fresh one (the benchmark's warm-up relies on this)."""
    base = Problem.from_deck(configs.sedov(16, kappa=0.01))
    pa, pb = base.copy(), base.copy()
    sa = Solver(pa, fp_mode=abi.FP_EXACT)
    init = {fid: a.copy() for fid, a in pa.fields.items()}
    ts0 = pa.timestep.copy()
    ierr, _ = sa.run(max_steps=5, ts=pa.timestep.copy(), history=False)
    assert ierr == 0
    for fid, a in init.items():
        np.copyto(pa.fields[fid], a)
    sa.sync_to_device(0)
    ta = ts0.copy()
    ierr, _ = sa.run(max_steps=30, ts=ta, history=False)
    assert ierr == 0, sa.error.message
    sb = Solver(pb, fp_mode=abi.FP_EXACT)
    tb = pb.timestep
    ierr, _ = sb.run(max_steps=30, ts=tb, history=False)
    assert ierr == 0
    assert (ta.nstep, ta.time, ta.dt) == (tb.nstep, tb.time, tb.dt)
    sa.sync_to_host(0)
    sb.sync_to_host(0)
    assert not compare(pa, pb, exact=True)


def test_hourglass_sedov_reaches_end_time():
    """The benchmark's workload at a small size: Sedov with the hourglass
    filter and sub-zonal pressures runs to t = 1 on the device loop, ending
    in the CPU restatement's state bit for bit."""
    from oracle.oracle import Oracle
    base = Problem.from_deck(configs.sedov(32, kappa=0.01, pmerit=0.1))
    pg, pc = base.copy(), base.copy()
    s = Solver(pg, fp_mode=abi.FP_EXACT)
    ierr, hist = s.run()
    assert ierr == 0, s.error.message
    assert pg.timestep.time >= 1.0
    s.sync_to_host(0)
    o = Oracle(pc)
    ierr, n = o.run(pc.timestep)
    assert ierr == 0 and n == len(hist)
    assert not compare(pg, pc, exact=True)


def test_fast_bench_workload_to_end_time():
    """Fast mode (the benchmark's mode) over the whole run of the benchmark's
    workload at 32x32: final totals and fields within the stated tolerances
    of the CPU restatement."""
    from oracle.oracle import Oracle
    base = Problem.from_deck(configs.sedov(32, kappa=0.01, pmerit=0.1))
    pg, pc = base.copy(), base.copy()
    s = Solver(pg, fp_mode=abi.FP_FAST)
    ierr, hist = s.run()
    assert ierr == 0, s.error.message
    s.sync_to_host(0)
    o = Oracle(pc)
    ierr, n = o.run(pc.timestep)
    assert ierr == 0 and n == len(hist)
    tg, tc = pg.totals(), pc.totals()
    assert abs(tg["mass"] - tc["mass"]) <= 1e-12 * abs(tc["mass"])
    et, ec = tg["ie"] + tg["ke"], tc["ie"] + tc["ke"]
    assert abs(et - ec) <= 1e-12 * abs(ec)
    for fid in (abi.ELDENSITY, abi.ELENERGY, abi.NDU, abi.NDV):
        a, b = pg.fields[fid], pc.fields[fid]
        l1 = np.sum(np.abs(a - b)) / max(np.sum(np.abs(b)), 1e-300)
        assert l1 <= 1e-9, (abi.NAMES[fid], l1)


def test_device_loop_step_limit_and_resume():
    base = Problem.from_deck(configs.noh(20, time_end=0.05, eulerian=True))
    pa, pb = base.copy(), base.copy()
    sa = Solver(pa, fp_mode=abi.FP_EXACT)
    ierr, h1 = sa.run(max_steps=7)
    assert ierr == 0 and len(h1) == 7
    ierr, h2 = sa.run(max_steps=40)
    assert ierr == 0
    sa.sync_to_host(0)
    sb = Solver(pb, fp_mode=abi.FP_EXACT)
    for _ in range(7 + len(h2)):
        assert sb.step() == 0
    sb.sync_to_host(0)
    assert not compare(pa, pb, exact=True)
    assert [r[0] for r in h1 + h2] == list(range(1, 8 + len(h2)))


def test_negative_volume_reports_element():
    """A tangled mesh returns ierr = -iel of the last bad element with
    HALT_SINGLE, like geometry_kn_checkvolume (fault made on the host)."""
    from oracle.oracle import Oracle
    p = Problem.from_deck(configs.sod(12, 3))
    # move one interior node across its right-hand neighbour (nodes are
    # numbered l + (k-1)*no_l with no_l = 4 here)
    k = 7 * 4 + 2
    p.fields[abi.NDX][k] += 2.5 * (1.0 / 12)
    pc = p.copy()
    s = Solver(p, fp_mode=abi.FP_EXACT)
    o = Oracle(pc)
    assert s.inf_solver_getdt() == o.getdt(pc.timestep)
    eg = s.inf_solver_lagstep()
    ec = o.lagstep(pc.timestep)
    assert eg == ec and eg < 0
    assert s.error.iout == abi.HALT_SINGLE
    assert "negative volume" in s.error.message


def test_dt_min_halt():
    deck = configs.sod(16, 4).replace("dt_min=1e-10", "dt_min=0.5").replace(
        "dt_max=0.001", "dt_max=1.0")
    p = Problem.from_deck(deck)
    s = Solver(p, fp_mode=abi.FP_EXACT)
    ierr = s.inf_solver_getdt()
    assert ierr == abi.FAILURE
    assert s.error.iout == abi.HALT_ALL
    assert s.error.message == "ERROR: dt < dt_min"
    assert p.timestep.nstep == 1   # time_dr_end updates before the check


def test_time_step_kernels_advances_like_the_device_loop():
    """bl_time_step_kernels (the per-kernel timing aid) runs the same
    kernels in the same order as bl_run: after 8 steps the state equals the
    device loop's bit for bit, and every kernel reports a positive time."""
    base = Problem.from_deck(configs.sedov(24, kappa=0.01, pmerit=0.1))
    pa, pb = base.copy(), base.copy()
    sa = Solver(pa, fp_mode=abi.FP_EXACT)
    ierr, ms = sa.time_step_kernels(8)
    assert ierr == 0, sa.error.message
    assert len(ms) == 4 and all(m > 0.0 for m in ms)
    sb = Solver(pb, fp_mode=abi.FP_EXACT)
    ierr, _ = sb.run(max_steps=8, history=False)
    assert ierr == 0
    assert (pa.timestep.nstep, pa.timestep.time, pa.timestep.dt) == (
        pb.timestep.nstep, pb.timestep.time, pb.timestep.dt)
    sa.sync_to_host(0)
    sb.sync_to_host(0)
    assert not compare(pa, pb, exact=True)
    ierr, _ = sa.time_step_kernels(65)
    assert ierr != 0 and "bad argument" in sa.error.message


def test_host_edits_of_the_timestep_take_effect():
    """The per-call entry points skip uploading the step header when the
    device already holds it; a host that edits the timestep between calls
    (dt, time, nstep) must still see its edit used, as the CPU restatement
    uses it."""
    from oracle.oracle import Oracle
    base = Problem.from_deck(configs.sedov(16, kappa=0.01, pmerit=0.1))
    pg, pc = base.copy(), base.copy()
    s = Solver(pg, fp_mode=abi.FP_EXACT)
    o = Oracle(pc)
    tg, tc = pg.timestep, pc.timestep
    for n in range(8):
        if n == 3:                 # edit between two steps
            for t in (tg, tc):
                t.dt = 0.5 * t.dt
                t.time = t.time + 1e-7
        assert s.inf_solver_getdt(tg) == o.getdt(tc) == 0
        if n == 5:                 # edit between getdt and lagstep
            for t in (tg, tc):
                t.dt = 0.75 * t.dt
        assert s.inf_solver_lagstep(tg) == o.lagstep(tc) == 0
        if n == 6:
            for t in (tg, tc):
                t.nstep = t.nstep + 10
        assert (tg.nstep, tg.dt, tg.time) == (tc.nstep, tc.dt, tc.time)
    s.sync_to_host(0)
    assert not compare(pg, pc, exact=True)


def test_sinusoidal_interface_halts_like_the_oracle():
    """The literal sinusoidal two-material Sod under the plain closure
    stops with dt < dt_min on the device at the same step and time as the
    CPU restatement (exact mode), well before t = 0.2."""
    from oracle.oracle import Oracle
    dk, fr = configs.sod_interface(200, 20, time_end=0.2)
    base = Problem.from_deck(dk, material_fraction=fr)
    pg, pc = base.copy(), base.copy()
    o = Oracle(pc)
    ierr_c, n_c = o.run(pc.timestep, 10**6)
    s = Solver(pg, fp_mode=abi.FP_EXACT)
    ierr_g, hist = s.run()
    assert ierr_c != 0 and ierr_g != 0
    assert s.error.message == "ERROR: dt < dt_min" == o.err.message.strip()
    assert pg.timestep.nstep == pc.timestep.nstep and pg.timestep.time == pc.timestep.time
    assert pg.timestep.time < 0.1
    s.close()
