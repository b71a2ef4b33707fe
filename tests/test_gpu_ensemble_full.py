"""The batched ensemble at its stated size: 512 seeded Eulerian Sod and
Sedov meshes of side logU(32, 512), 22.6M elements in one batch.  The
oracle cannot run the whole ensemble, so parity is shown by properties
that do not depend on its size: after the first steps of the batch in
exact mode, every mesh equals the same mesh run alone through the
per-mesh device loop, bit for bit (state and timestep record), and a
sample of meshes (the smallest and largest of each kind) equals the
oracle bit for bit."""
import numpy as np
import pytest

from bookleaf_f90_gb300 import BatchSolver, Problem, Solver, abi, configs
from helpers import compare

pytestmark = pytest.mark.gpu

STEPS = 10


def _same_timestep(a, b):
    return ((a.nstep, a.time, a.dt, a.idtel, bytes(a.sdt)) ==
            (b.nstep, b.time, b.dt, b.idtel, bytes(b.sdt)))


def test_full_ensemble_first_steps_equal_each_mesh_and_the_oracle():
    from oracle.oracle import Oracle
    ens = configs.ensemble(512)
    probs = [Problem.from_deck(d) for d, _ in ens]
    assert sum(p.nel for p in probs) > 2.0e7
    # the sample for the oracle: smallest and largest Sod and Sedov meshes
    kinds = [m["kind"] for _, m in ens]
    sample = set()
    for k in ("sod", "sedov"):
        idx = [i for i in range(len(ens)) if kinds[i] == k]
        sample.add(min(idx, key=lambda i: probs[i].nel))
        sample.add(max(idx, key=lambda i: probs[i].nel))
    refs = {i: probs[i].copy() for i in sample}
    b = BatchSolver(probs, fp_mode=abi.FP_EXACT)
    ierr, status, n = b.run(max_steps=STEPS)
    assert ierr == 0 and n == STEPS and status == [0] * len(probs), b.error.message
    b.sync_to_host(0)
    b.close()
    for i, (deck, _) in enumerate(ens):
        q = Problem.from_deck(deck)
        s = Solver(q, fp_mode=abi.FP_EXACT)
        ierr, _ = s.run(max_steps=STEPS, history=False)
        assert ierr == 0, s.error.message
        s.sync_to_host(0)
        s.close()
        assert _same_timestep(probs[i].timestep, q.timestep), i
        bad = compare(probs[i], q, exact=True, where="mesh %d" % i)
        assert not bad, bad[:3]
    for i, r in refs.items():
        o = Oracle(r)
        ts = r.timestep
        for _ in range(STEPS):
            assert o.step(ts) == 0, o.err.message
        assert _same_timestep(probs[i].timestep, ts), i
        bad = compare(probs[i], r, exact=True, where="mesh %d vs oracle" % i)
        assert not bad, bad[:3]
    assert len({probs[i].nel for i in sample}) == len(sample)
    assert np.isfinite(sum(p.totals()["mass"] for p in probs))
