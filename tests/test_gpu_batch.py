"""A batch of independent problems (bl_init_batch / bl_run_batch) advances
every mesh as it would alone: each mesh's final fields and timestep equal
those of running it by itself with the device loop, bit for bit, in exact
and in fast mode.  The meshes differ in size, gamma, pressure ratio,
time-step controls and end time, so they take different dt sequences and
finish at different steps."""
import ctypes as ct

import pytest

from bookleaf_f90_gb300 import BatchSolver, Problem, Solver, SolverError, abi, configs
from helpers import compare

pytestmark = pytest.mark.gpu

LAGRANGIAN = [
    configs.sod(24, 4, time_end=0.05),
    configs.sedov(16, time_end=0.02),
    configs.sod(30, 3, time_end=0.03, gamma=1.6, pratio=100.0),
    configs.sedov(12, time_end=0.05, gamma=1.25),
]
EULERIAN = [
    configs.sod(20, 4, time_end=0.03, eulerian=True),
    configs.sedov(14, time_end=0.02, eulerian=True, gamma=1.6),
    configs.sod(16, 2, time_end=0.02, eulerian=True, gamma=1.3, pratio=1000.0),
]


def _alone(deck, fp):
    p = Problem.from_deck(deck)
    s = Solver(p, fp_mode=fp)
    ierr, _ = s.run(history=False)
    s.sync_to_host(0)
    s.close()
    return ierr, p


def _same_timestep(a, b):
    return ((a.nstep, a.time, a.dt, a.idtel, bytes(a.sdt), a.imdt) ==
            (b.nstep, b.time, b.dt, b.idtel, bytes(b.sdt), b.imdt))


@pytest.mark.parametrize("fp", [abi.FP_EXACT, abi.FP_FAST], ids=["exact", "fast"])
@pytest.mark.parametrize("decks", [LAGRANGIAN, EULERIAN], ids=["lagrangian", "eulerian"])
def test_batch_equals_each_mesh_alone(decks, fp):
    probs = [Problem.from_deck(d) for d in decks]
    b = BatchSolver(probs, fp_mode=fp)
    ierr, status, nsteps = b.run()
    assert ierr == 0 and status == [0] * len(decks), b.error.message
    b.sync_to_host(0)
    steps = []
    for d, p in zip(decks, probs):
        ierr1, q = _alone(d, fp)
        assert ierr1 == 0
        assert _same_timestep(p.timestep, q.timestep), (p.timestep.as_tuple(), q.timestep.as_tuple())
        assert not compare(p, q, exact=True)
        steps.append(p.timestep.nstep)
    assert len(set(steps)) > 1          # the meshes really ran different step counts
    assert max(steps) <= nsteps < max(steps) + 16
    b.close()


@pytest.mark.parametrize("decks", [LAGRANGIAN, EULERIAN], ids=["lagrangian", "eulerian"])
def test_compacting_run_equals_each_mesh_alone(decks):
    """run_compacting rebuilds the batch from the meshes still running
    (their state through the host) whenever they hold less than `keep` of
    the elements; with chunks of 8 steps and keep 0.9 it rebuilds several
    times, and every mesh still ends bit for bit as alone."""
    probs = [Problem.from_deck(d) for d in decks]
    b = BatchSolver(probs, fp_mode=abi.FP_EXACT)
    ierr, status, nsteps = b.run_compacting(keep=0.9, chunk=8)
    assert ierr == 0 and all(v == 0 for v in status.values()), b.error.message
    b.sync_to_host(0)
    assert len(b.compactions) >= 1
    assert b.total_launches > 0
    b.close()
    for d, p in zip(decks, probs):
        ierr1, q = _alone(d, abi.FP_EXACT)
        assert ierr1 == 0
        assert _same_timestep(p.timestep, q.timestep), (p.timestep.as_tuple(), q.timestep.as_tuple())
        assert not compare(p, q, exact=True)


def test_batch_step_limit_then_resume():
    """A run stopped after k steps and resumed ends where one run ends."""
    probs = [Problem.from_deck(d) for d in LAGRANGIAN]
    b = BatchSolver(probs, fp_mode=abi.FP_EXACT)
    ierr, status, n1 = b.run(max_steps=21)
    assert ierr == 0 and n1 == 21
    assert all(p.timestep.nstep <= 21 for p in probs)
    ierr, status, n2 = b.run()
    assert ierr == 0, b.error.message
    b.sync_to_host(0)
    for d, p in zip(LAGRANGIAN, probs):
        _, q = _alone(d, abi.FP_EXACT)
        assert _same_timestep(p.timestep, q.timestep)
        assert not compare(p, q, exact=True)


def test_failing_mesh_reports_its_status_and_leaves_the_others():
    """A mesh that stops on dt < dt_min reports it in its own status; the
    other meshes of the batch run on to their end times unchanged."""
    bad = configs.sod(16, 4, time_end=0.05).replace("dt_min=1e-10", "dt_min=0.5").replace(
        "dt_max=0.001", "dt_max=1.0")
    decks = [LAGRANGIAN[0], bad, LAGRANGIAN[1]]
    probs = [Problem.from_deck(d) for d in decks]
    b = BatchSolver(probs, fp_mode=abi.FP_EXACT)
    ierr, status, _ = b.run()
    assert ierr != 0 and status == [0, abi.FAILURE, 0]
    assert "mesh 2" in b.error.message and "dt < dt_min" in b.error.message
    b.sync_to_host(0)
    for i in (0, 2):
        _, q = _alone(decks[i], abi.FP_EXACT)
        assert _same_timestep(probs[i].timestep, q.timestep)
        assert not compare(probs[i], q, exact=True)


def test_batch_rejects_different_settings_and_single_mesh_calls():
    with pytest.raises(SolverError, match="settings differ"):
        BatchSolver([Problem.from_deck(LAGRANGIAN[0]), Problem.from_deck(EULERIAN[0])])
    probs = [Problem.from_deck(d) for d in LAGRANGIAN[:2]]
    b = BatchSolver(probs, fp_mode=abi.FP_EXACT)
    assert b.L.bl_batch_size(b.ctx) == 2
    err = abi.Error()
    ts = probs[0].timestep
    assert b.L.bl_getdt(b.ctx, ct.byref(ts), ct.byref(err)) == abi.FAILURE
    assert "batch context" in err.message
    b.close()


def test_autotuned_batch_still_equals_each_mesh_alone():
    """The autotuner runs candidates from the registered host arrays and
    uploads them again: the run after it is unchanged, bit for bit."""
    probs = [Problem.from_deck(d) for d in EULERIAN]
    b = BatchSolver(probs, fp_mode=abi.FP_EXACT)
    g, bs, ms = b.autotune()
    assert g in (8, 16, 32) and bs in (128, 256, 512)
    assert all(v > 0.0 for v in ms.values()) and ms[(g, bs)] == min(ms.values())
    ierr, status, _ = b.run()
    assert ierr == 0, b.error.message
    b.sync_to_host(0)
    for d, p in zip(EULERIAN, probs):
        _, q = _alone(d, abi.FP_EXACT)
        assert _same_timestep(p.timestep, q.timestep)
        assert not compare(p, q, exact=True)
    b.close()


# two-material tubes (mixed cells along a tilted interface) of different
# sizes, tilts and states, and a pure Sod tube
def _two_material(nx, tilt, st, time_end=0.02):
    deck, frac = configs.sod_interface(nx, nx // 10, time_end=time_end, amplitude=0.0, periods=0,
                                       tilt=tilt, rho_right=st, p_right=st)
    return Problem.from_deck(deck, material_fraction=frac)


def _mixed_problems():
    return [_two_material(80, 0.2, 0.5), _two_material(64, 0.3, 0.6, 0.015),
            Problem.from_deck(configs.sod(24, 4, time_end=0.02)),
            _two_material(96, 0.1, 0.4, 0.025)]


def _closure_net():
    from bookleaf_f90_gb300 import closure
    import numpy as np
    # an untrained network: its exchanges are arbitrary, within the
    # admissible range, which is all the batch comparison needs
    net = closure.ClosureNet(seed=3)
    norm = np.concatenate([[0.5, 1, 0.5, 1, 0.5, 1.4, 1.5, 0, 0.1, 0.3],
                           [3, 2, 3, 2, 3, 2, 2, 300, 5, 2], [1e-3, 10.0]])
    return net, norm


@pytest.mark.parametrize("learned", [False, True], ids=["plain", "learned"])
@pytest.mark.parametrize("fp", [abi.FP_EXACT, abi.FP_FAST], ids=["exact", "fast"])
def test_batch_with_mixed_cells_equals_each_mesh_alone(fp, learned):
    """Meshes with mixed cells concatenate with their component and
    mixed-cell numbers offset; under the plain or the learned closure each
    ends as it does alone, bit for bit, and the closure sees the same cells."""
    net, norm = _closure_net() if learned else (None, None)
    probs = _mixed_problems()
    b = BatchSolver(probs, fp_mode=fp)
    if learned:
        b.set_closure(net, norm)
    ierr, status, _ = b.run()
    assert ierr == 0 and status == [0] * len(probs), b.error.message
    b.sync_to_host(0)
    seen_b = b.closure_stats()
    b.close()
    seen = [0, 0]
    for i, q in enumerate(_mixed_problems()):
        s = Solver(q, fp_mode=fp)
        if learned:
            s.set_closure(net, norm)
        ierr, _ = s.run(history=False)
        assert ierr == 0, s.error.message
        s.sync_to_host(0)
        st = s.closure_stats()
        seen[0] += st[0]
        seen[1] += st[1]
        s.close()
        p = probs[i]
        assert _same_timestep(p.timestep, q.timestep), (i, p.timestep.as_tuple(), q.timestep.as_tuple())
        assert not compare(p, q, exact=True), i
        if q.sizes.ncp:
            for fid in (abi.CPVOLUME, abi.CPENERGY, abi.CPDENSITY, abi.FRVOLUME):
                assert (p.fields[fid] == q.fields[fid]).all(), (i, abi.NAMES[fid])
    assert tuple(seen) == seen_b
    if learned:
        assert seen_b[0] > 0 and seen_b[1] < seen_b[0]
        net.close()
