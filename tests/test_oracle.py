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


def test_elementary_functions_follow_the_c_library():
    """exp, log and pow of the equations of state (orc_exp/orc_log/orc_pow,
    the same operations as the device's bl_exp/bl_log/bl_pow): within one
    unit in the last place of the C library's for exp and pow, two for log,
    and equal to it for most arguments; IEEE special cases."""
    import ctypes as ct
    import math
    from oracle import oracle as orc
    L = ct.CDLL(orc.build())
    for n in ("orc_exp", "orc_log"):
        getattr(L, n).restype = ct.c_double
        getattr(L, n).argtypes = [ct.c_double]
    L.orc_pow.restype = ct.c_double
    L.orc_pow.argtypes = [ct.c_double, ct.c_double]
    rng = np.random.default_rng(3)

    def ulps(got, ref):
        return 0.0 if got == ref else abs(got - ref) / math.ulp(ref)

    cases = [("exp", 1.0, lambda x, y: L.orc_exp(x), lambda x, y: math.exp(x),
              rng.uniform(-700, 700, 4000), None),
             ("log", 2.0, lambda x, y: L.orc_log(x), lambda x, y: math.log(x),
              np.exp(rng.uniform(-700, 700, 4000)), None),
             ("pow", 1.0, lambda x, y: L.orc_pow(x, y), lambda x, y: math.pow(x, y),
              rng.uniform(0.01, 100, 4000), rng.uniform(-10, 10, 4000))]
    for name, bound, f, g, xs, ys in cases:
        ys = ys if ys is not None else np.zeros_like(xs)
        u = np.array([ulps(f(float(x), float(y)), g(float(x), float(y))) for x, y in zip(xs, ys)])
        assert u.max() <= bound, (name, u.max())
        assert np.mean(u == 0) > 0.7, (name, np.mean(u == 0))
    assert L.orc_exp(0.0) == 1.0 and L.orc_log(1.0) == 0.0
    assert L.orc_pow(1.0, 7.15) == 1.0 and L.orc_pow(3.0, 0.0) == 1.0
    assert L.orc_pow(0.0, 2.0) == 0.0 and L.orc_exp(-800.0) == 0.0
    assert math.isinf(L.orc_exp(800.0)) and math.isnan(L.orc_pow(-1.0, 0.5))


@pytest.mark.parametrize("form", ["void", "tait", "jwl"])
def test_other_eos_forms_conserve(form):
    """The two-material tubes with a void, Tait or JWL material: the
    restatement runs them, masses are unchanged and total energy is kept to
    round-off; the Tait tube reaches its pressure floor."""
    deck = configs.eos_tube(form, 60, 6)
    p0 = Problem.from_deck(deck)
    assert p0.config.eos_type[2] == {"void": 0, "tait": 2, "jwl": 3}[form]
    assert p0.sizes.nmx > 0
    t0 = p0.totals()
    p, n = run(deck, 100)
    t1 = p.totals()
    assert t1["mass"] == t0["mass"]
    e0, e1 = t0["ie"] + t0["ke"], t1["ie"] + t1["ke"]
    assert abs(e1 - e0) <= 1e-12 * abs(e0) * n
    if form == "tait":
        assert np.any(p.fields[abi.ELPRESSURE] == -0.1)


def test_plain_closure_halts_on_the_sinusoidal_interface():
    """The two-material Sod with the sinusoidal interface (amplitude 0.02,
    8 periods) cannot be run to t = 0.2 under the reference's plain
    closure: its mixed cells get neither artificial viscosity nor
    hourglass control, collapse, and the step ends with dt < dt_min
    (HALT_ALL) at t ~ 0.05 on 200x20.  The learned closure's measurements
    therefore use a tilted planar interface the plain closure survives."""
    dk, fr = configs.sod_interface(200, 20, time_end=0.2)
    p = Problem.from_deck(dk, material_fraction=fr)
    assert p.sizes.nmx > 100
    o = Oracle(p)
    ierr, n = o.run(p.timestep, 10**6)
    assert ierr != 0 and o.err.message.strip() == "ERROR: dt < dt_min"
    assert p.timestep.time < 0.1
