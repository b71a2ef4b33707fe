"""bl_init's checks of the connectivity, which run on the device
(csrc/bl_setup.cuh): each error class is reported with its message, in the
order of precedence of the host checks they replaced, a rejected set-up
leaves the device usable, and the device-built node -> corner tables
follow a shuffled ielsort1 as the oracle does, bit for bit."""
import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, Solver, SolverError, abi, configs
from bookleaf_f90_gb300.setup import mesh as meshmod

pytestmark = pytest.mark.gpu


def _sod():
    return Problem.from_deck(configs.sod(16, 4))


def _reject(p):
    with pytest.raises(SolverError) as ex:
        Solver(p)
    return str(ex.value)


def _plant(p, fid, where, value):
    p.fields[fid][where] = value


CASES = [
    ("node above nnd", abi.IELND, (3, 1), lambda p: p.nnd + 1, "connectivity out of range"),
    ("node zero", abi.IELND, (3, 1), lambda p: 0, "connectivity out of range"),
    ("neighbour above nel", abi.IELEL, (5, 2), lambda p: p.nel + 1, "connectivity out of range"),
    ("face 5", abi.IELFC, (5, 0), lambda p: 5, "connectivity out of range"),
    ("region above nreg", abi.IELREG, (7,), lambda p: p.sizes.nreg + 1,
     "ielreg/ielsort1 out of range"),
    ("sort position zero", abi.IELSORT1, (7,), lambda p: 0, "ielreg/ielsort1 out of range"),
    ("sort position repeated", abi.IELSORT1, (7,), lambda p: int(p.fields[abi.IELSORT1][8]),
     "ielsort1 is not a permutation"),
    ("material above nmat", abi.IELMAT, (9,), lambda p: p.sizes.nmat + 1,
     "ielmat out of range"),
]


@pytest.mark.parametrize("name,fid,where,value,msg", CASES, ids=[c[0] for c in CASES])
def test_each_error_class_is_reported(name, fid, where, value, msg):
    p = _sod()
    _plant(p, fid, where, value(p))
    assert msg in _reject(p)


def test_connectivity_error_takes_precedence():
    p = _sod()
    _plant(p, abi.IELMAT, (9,), p.sizes.nmat + 1)
    _plant(p, abi.IELSORT1, (7,), 0)
    _plant(p, abi.IELND, (3, 1), p.nnd + 1)
    assert "connectivity out of range" in _reject(p)
    p = _sod()
    _plant(p, abi.IELMAT, (9,), p.sizes.nmat + 1)
    _plant(p, abi.IELSORT1, (7,), int(p.fields[abi.IELSORT1][8]))
    assert "not a permutation" in _reject(p)


def test_rejected_setup_leaves_the_device_usable():
    bad = _sod()
    _plant(bad, abi.IELEL, (5, 2), bad.nel + 1)
    _reject(bad)
    p = _sod()
    s = Solver(p, fp_mode=abi.FP_EXACT)
    ierr, _ = s.run(max_steps=5, history=False)
    assert ierr == 0, s.error.message
    s.close()


def _rotate_corners(monkeypatch, seed=5):
    """Make Problem.from_deck rotate each element's node list by a seeded
    cyclic shift before the connectivity and the initial state are derived
    from it: still a counter-clockwise mesh, but a node can now be the same
    corner of several elements, and then ielsort1 orders them."""
    gen0 = meshmod.generate

    def gen(*a, **k):
        out = list(gen0(*a, **k))
        ielnd = out[3]
        r = np.random.default_rng(seed).integers(0, 4, len(ielnd))
        idx = (np.arange(4)[None, :] + r[:, None]) % 4
        out[3] = np.ascontiguousarray(np.take_along_axis(ielnd, idx, axis=1))
        return tuple(out)

    monkeypatch.setattr(meshmod, "generate", gen)


def _oracle_final(p, steps):
    from oracle.oracle import Oracle
    o = Oracle(p)
    ts = p.timestep
    for _ in range(steps):
        assert o.getdt(ts) == 0 and o.lagstep(ts) == 0 and o.alestep(ts) == 0
    return np.concatenate([p.fields[abi.NDU], p.fields[abi.ELENERGY]])


SHUFFLED = [("sedov_24", lambda: configs.sedov(24, kappa=0.01, pmerit=0.1), 8),
            ("sedov_24_eulerian", lambda: configs.sedov(24, eulerian=True), 20)]


@pytest.mark.parametrize("name,deck,steps", SHUFFLED, ids=[c[0] for c in SHUFFLED])
def test_shuffled_ielsort1_matches_the_oracle(monkeypatch, name, deck, steps):
    """ielsort1 orders the corners of a node that are the same corner of
    several elements in the nodal acceleration gather
    (hydro_kn_getacceleration.f90:53-72); the device-built tables must
    follow it.  On a mesh with rotated corner numbering and a seeded random
    ielsort1, the run must equal the oracle's bit for bit, and the oracle's
    own bits must depend on that order (so that the case tests it)."""
    from helpers import run_pair
    _rotate_corners(monkeypatch)
    p = Problem.from_deck(deck())
    ident = _oracle_final(p.copy(), steps)
    p.fields[abi.IELSORT1][...] = np.random.default_rng(11).permutation(p.nel) + 1
    pg, pc, bad = run_pair(p, steps, exact=True, phases=False)
    assert not bad, bad[:3]
    assert not np.array_equal(ident, np.concatenate([pc.fields[abi.NDU],
                                                     pc.fields[abi.ELENERGY]]))
