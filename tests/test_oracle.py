"""The CPU restatement (test infrastructure) against the reference's own
known-answer test and conservation invariants, plus regression fixtures.

The reference ships no golden vectors.  Its one known-answer test is the
Sod L1 density norm against the exact Riemann solution
(src/packages/check/kernel/check_kn_tests.f90:33-111), printed at run end
for decks whose file name contains "sod" (check_dr_validate.f90:74-78).
"""
import json
import os

import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, abi, configs
from oracle.oracle import Oracle, sod_l1

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def run(deck, max_steps=10**9):
    p = Problem.from_deck(deck)
    o = Oracle(p)
    ierr, n = o.run(p.timestep, max_steps)
    assert ierr == 0, o.err.message
    return p, n


def test_sod_known_answer_reference_geometry():
    """The reference's check geometry: x in [0,100], interface 50, t=20."""
    p, n = run(configs.sod_reference(100, 10, time_end=20.0))
    l1_rho, l1_e = sod_l1(p, p.timestep.time)
    # first-order shock capturing on 100 cells: a few 1e-3
    assert 1.0e-3 < l1_rho < 1.0e-2
    assert l1_e < 5.0e-2
    # refining halves the error (convergence of the restated scheme)
    p2, _ = run(configs.sod_reference(200, 4, time_end=20.0))
    l1_rho2, _ = sod_l1(p2, p2.timestep.time)
    assert l1_rho2 < 0.7 * l1_rho


def test_sod_reference_deck():
    """The reference's own Sod deck (input/sod_sm_lag_small, vendored under
    tests/golden/decks): density L1 against the exact solution as
    check_dr_validate prints it."""
    import golden
    p, n = run(golden.deck_text("sod_sm_lag_small"))
    l1, _ = sod_l1(p, p.timestep.time)
    assert 1.0e-3 < l1 < 1.0e-2


@pytest.mark.parametrize("deck", [configs.sedov(24, time_end=0.05), configs.noh(20, time_end=0.05)])
def test_lagrangian_conservation(deck):
    p0 = Problem.from_deck(deck)
    t0 = p0.totals()
    p, n = run(deck)
    t1 = p.totals()
    assert t1["mass"] == t0["mass"]                      # masses never change
    e0, e1 = t0["ie"] + t0["ke"], t1["ie"] + t1["ke"]
    assert abs(e1 - e0) <= 1e-12 * max(abs(e0), 1e-30) * n


def test_eulerian_mass_conservation_closed_box():
    """Sod in a closed box remapped every step keeps its mass."""
    deck = configs.sod(40, 4, time_end=0.02, eulerian=True)
    p0 = Problem.from_deck(deck)
    m0 = p0.fields[abi.ELMASS].sum()
    p, n = run(deck)
    m1 = p.fields[abi.ELMASS].sum()
    assert abs(m1 - m0) <= 1e-12 * m0
    # the mesh returns to the initial Eulerian mesh
    assert np.allclose(p.fields[abi.NDX], p0.fields[abi.NDX], atol=1e-12)


def test_regression_fixtures():
    """Fixtures written by tests/golden/make_golden.py from this restatement:
    they pin the restatement against accidental change."""
    with open(os.path.join(GOLDEN, "oracle_runs.json")) as f:
        gold = json.load(f)
    from golden.make_golden import CASES, summarise
    for name, (deck, steps) in CASES.items():
        p, _ = run(deck, steps)
        got = summarise(p)
        ref = gold[name]
        for k, v in ref.items():
            assert got[k] == v, (name, k, got[k], v)


def test_fixture_checksum_sees_every_element():
    """The fixtures' checksum changes when any element changes, including
    arrays whose values all occur an even number of times, and the stored
    fixtures hold no two equal checksums of different fields."""
    from golden.make_golden import _bits
    a = np.repeat(np.arange(10.0), 4)
    b = np.repeat(np.arange(10.0) + 1, 4)
    assert _bits(a) != _bits(b)
    c = a.copy()
    c[[3, 4]] = c[[4, 3]]
    assert _bits(c) != _bits(a[::-1])
    d = a.copy()
    d[17] = np.nextafter(d[17], 1e9)
    assert _bits(d) != _bits(a)
    assert _bits(np.zeros(8)) != _bits(np.zeros(16))
    with open(os.path.join(GOLDEN, "oracle_runs.json")) as f:
        gold = json.load(f)
    for name, rec in gold.items():
        sums = [v for k, v in rec.items() if isinstance(v, str)]
        assert len(sums) == len(set(sums)), name
