"""Side-by-side drivers for the GPU path and the CPU restatement."""
import numpy as np

from bookleaf_f90_gb300 import Problem, Solver, abi, configs  # noqa: F401

# Fields a host reader sees between solver calls (bl_sync_to_host(ctx, 0)).
STATE = [abi.ELDENSITY, abi.ELENERGY, abi.ELPRESSURE, abi.ELCS2, abi.ELVOLUME, abi.A1,
         abi.A2, abi.A3, abi.B1, abi.B2, abi.B3, abi.CNWT, abi.CNX, abi.CNY, abi.CNVISCX,
         abi.CNVISCY, abi.ELVISC, abi.ELMASS, abi.CNMASS, abi.NDX, abi.NDY, abi.NDU, abi.NDV]
CPSTATE = [abi.CPDENSITY, abi.CPENERGY, abi.CPPRESSURE, abi.CPCS2, abi.CPVOLUME,
           abi.CPA1, abi.CPA3, abi.CPB1, abi.CPB3]


def state_ids(p):
    return STATE + (CPSTATE if p.sizes.ncp > 0 else [])


def compare(pg, pc, exact, rtol=1e-11, atol=1e-14, where=""):
    """Compare every state field of two problems; return list of mismatches."""
    bad = []
    for fid in state_ids(pg):
        a = pg.fields.get(fid)
        b = pc.fields.get(fid)
        if a is None or b is None:
            continue
        if exact:
            if not np.array_equal(a, b):
                d = np.nonzero(~((a == b) | (np.isnan(a) & np.isnan(b))))
                if len(d[0]):
                    i = tuple(x[0] for x in d)
                    bad.append("%s %s: first diff at %s gpu=%r cpu=%r (%d diffs)"
                               % (where, abi.NAMES[fid], i, a[i], b[i], len(d[0])))
        else:
            if not np.allclose(a, b, rtol=rtol, atol=atol):
                err = np.max(np.abs(a - b) / (np.abs(b) + atol))
                bad.append("%s %s: max rel err %.3e" % (where, abi.NAMES[fid], err))
    return bad


def run_pair(deck, nsteps, exact=True, phases=True, rtol=1e-11, atol=1e-14):
    """Step the GPU (C-ABI) and the oracle side by side; compare after each
    phase when `phases`, else at the end.  Returns (gpu problem, cpu
    problem, list of mismatches)."""
    from oracle.oracle import Oracle
    base = Problem.from_deck(deck) if isinstance(deck, str) else deck
    pg, pc = base.copy(), base.copy()
    s = Solver(pg, fp_mode=abi.FP_EXACT if exact else abi.FP_FAST)
    o = Oracle(pc)
    tg, tc = pg.timestep, pc.timestep
    bad = []
    for n in range(nsteps):
        for name, fg, fc in (("getdt", s.inf_solver_getdt, o.getdt),
                             ("lagstep", s.inf_solver_lagstep, o.lagstep),
                             ("alestep", s.inf_solver_alestep, o.alestep)):
            eg = fg(tg)
            ec = fc(tc)
            if eg != ec:
                bad.append("step %d %s: ierr gpu=%d cpu=%d (%s / %s)" % (
                    n + 1, name, eg, ec, s.error.message, o.err.message))
                return pg, pc, bad
            if (tg.nstep, tg.dt, tg.time, tg.idtel, tg.sdt) != (tc.nstep, tc.dt, tc.time,
                                                              tc.idtel, tc.sdt):
                bad.append("step %d %s: timestep gpu=%s cpu=%s" % (
                    n + 1, name, tg.as_tuple(), tc.as_tuple()))
                return pg, pc, bad
            if eg != 0:
                return pg, pc, bad
            if phases:
                s.sync_to_host(0)
                bad += compare(pg, pc, exact, rtol, atol, "step %d %s" % (n + 1, name))
                if bad:
                    return pg, pc, bad
    s.sync_to_host(0)
    bad += compare(pg, pc, exact, rtol, atol, "final")
    s.close()
    return pg, pc, bad
