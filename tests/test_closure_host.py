"""Host side of the learned closure (bookleaf_f90_gb300/closure.py): the
sub-cell aggregation, the features and the standardisation the device
kernel reads.  No GPU."""
import numpy as np

from bookleaf_f90_gb300 import Problem, abi, closure, configs


def _problem(nx, ny):
    deck, frac = configs.sod_interface(nx, ny, time_end=0.01)
    return Problem.from_deck(deck, material_fraction=frac)


def test_parameter_layout():
    p = closure.init_params(3)
    assert p.dtype == np.float32 and p.size == closure.NPARAM == abi_nparam()
    # biases start at zero: b1 after W1, b2 after W2, b3 last
    nh, ni, no = closure.NH, closure.NI, closure.NO
    assert not np.any(p[nh * ni:nh * ni + nh])
    assert not np.any(p[-no:])


def abi_nparam():
    import os
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                       "bookleaf_gb300.h")
    return int(re.search(r"#define BL_MLP_NPARAM (\d+)", open(hdr).read()).group(1))


def test_fine_material_sums_add_up_to_the_coarse_cells():
    """Aggregating a 4x-refined mesh over the coarse grid gives each coarse
    cell the material volumes and masses the coarse mesh itself holds (to
    the accuracy of the area fractions' quadrature, whose integrand has
    kinks where the interface leaves a cell)."""
    nx, ny = 40, 4
    pc, pf = _problem(nx, ny), _problem(4 * nx, 4 * ny)
    Vc, Mc, Ec = closure.material_sums(pc, closure.grid_index(pc, nx, ny), nx * ny)
    Vf, Mf, Ef = closure.material_sums(pf, closure.grid_index(pf, nx, ny), nx * ny)
    vol = 1.0 / nx * 0.1 / ny
    assert np.allclose(Vf, Vc, rtol=0, atol=1e-5 * vol)
    assert np.allclose(Mf, Mc, rtol=0, atol=1e-5 * vol)
    assert np.allclose(Ef, Ec, rtol=0, atol=3e-5 * vol)
    assert abs(Vc[:, 1].sum() - 0.05) < 1e-12 and abs(Vc.sum() - 0.1) < 1e-12
    assert pc.sizes.nmx == int(np.sum((Vc[:, 0] > 0) & (Vc[:, 1] > 0)))


def test_features_of_the_initial_interface_cells():
    nx, ny = 40, 4
    p = _problem(nx, ny)
    V, M, E = closure.material_sums(p, closure.grid_index(p, nx, ny), nx * ny)
    mixed = (V[:, 0] > 0) & (V[:, 1] > 0)
    X = closure.features(p.config, V[mixed], M[mixed], E[mixed], np.zeros(mixed.sum()), 1e-3)
    assert X.shape == (mixed.sum(), closure.NI)
    g2 = 1.67
    assert np.allclose(X[:, 1], 1.0) and np.allclose(X[:, 2], 0.125)
    assert np.allclose(X[:, 3], 1.0) and np.allclose(X[:, 4], 0.1)
    assert np.allclose(X[:, 5], 1.4) and np.allclose(X[:, 6], g2 * 0.1 / 0.125)
    assert np.allclose(X[:, 0], V[mixed, 0] / V[mixed].sum(axis=1))
    cell = V[mixed].sum(axis=1)
    assert np.allclose(X[:, 8], 1e-3 * np.sqrt(1.4 / cell))     # max(1.4, 1.336)
    assert np.allclose(X[:, 9], 0.9 / 1.1)


def test_standardisation_and_exchange():
    rng = np.random.default_rng(0)
    X = rng.normal([0.5, 2, 3, 4, 5, 6, 7, 0, 9, 10], [0.1, 2, 3, 4, 5, 6, 7, 1e-3, 9, 0],
                   (500, 10))
    x1 = rng.normal(0, 2e-4, 500)
    fr = np.stack([X[:, 0], 1.0 - X[:, 0]], axis=1)
    D = fr * X[:, 7:8] + np.stack([x1, -x1], axis=1)      # plain share + exchange
    norm = closure.fit_norm(X, D)
    assert norm.shape == (2 * closure.NI + 2,) and norm.dtype == np.float32
    assert np.allclose(closure.exchange(X, D), np.stack([x1, -x1], axis=1), atol=1e-15)
    assert abs(norm[20] - np.sqrt(np.mean(x1 ** 2))) < 1e-6 * norm[20]
    x, t = closure.standardise(X, D, norm)
    assert np.allclose(x[:, :9].mean(axis=0), 0, atol=1e-5)
    assert np.allclose(x[:, :9].std(axis=0), 1, atol=1e-4)
    assert np.all(x[:, 9] == 0) and norm[19] == 1.0       # a constant feature
    assert np.allclose(t * norm[20], np.stack([x1, -x1], axis=1), rtol=1e-5, atol=1e-12)


def test_closure_step_restatement_conserves_volume_and_energy(oracle_lib):
    """One closure step on the CPU (oracle/closure.py) after 30 oracle steps:
    each accepted cell's material volumes still add up to the cell's, the
    fractions to 1, the energy moved between its materials sums to zero
    (exchange mode) or no energy moves (volume only), and masses stay."""
    from oracle import closure as oclosure
    from oracle.oracle import Oracle
    from bookleaf_f90_gb300.setup import ic as icmod
    deck, frac = configs.sod_interface(80, 8, time_end=0.2, amplitude=0.0, periods=0, tilt=0.2,
                                       rho_right=0.5, p_right=0.5)
    p = Problem.from_deck(deck, material_fraction=frac)
    o = Oracle(p)
    for _ in range(30):
        assert o.step(p.timestep) == 0
    f = p.fields
    nmx = p.sizes.nmx
    el = f[abi.IMXEL][:nmx] - 1
    c0 = f[abi.IMXFCP][:nmx] - 1
    before = {"frvol": f[abi.FRVOLUME].copy(), "cprho": f[abi.CPDENSITY].copy(),
              "cpp": f[abi.CPPRESSURE].copy(), "cpcs2": f[abi.CPCS2].copy(),
              "vol0": f[abi.ELVOLUME][el].copy()}
    assert o.step(p.timestep) == 0
    params = closure.init_params(5)
    norm = np.concatenate([[0.5, 1, 0.5, 1, 0.5, 1.4, 1.5, 0, 0.1, 0.3],
                           [3, 2, 3, 2, 3, 2, 2, 300, 5, 2], [1e-3, 10.0]]).astype(np.float32)
    energy = lambda g: g[abi.CPMASS][c0] * g[abi.CPENERGY][c0] + \
        g[abi.CPMASS][c0 + 1] * g[abi.CPENERGY][c0 + 1]
    for mode in (1, 2):
        g = {k: v.copy() for k, v in f.items()}
        ok = oclosure.apply(g, before, p.timestep.dt, params, norm, mode,
                            lambda m, r, e: icmod.eos(p.config, m, r, e), p.config.zerocut)
        assert ok.sum() > 0
        V1 = g[abi.ELVOLUME][el]
        assert np.allclose(g[abi.CPVOLUME][c0] + g[abi.CPVOLUME][c0 + 1], V1, rtol=1e-13, atol=0)
        assert np.allclose(g[abi.FRVOLUME][c0] + g[abi.FRVOLUME][c0 + 1], 1.0, rtol=0, atol=1e-13)
        assert np.allclose(energy(g), energy(f), rtol=1e-12, atol=0)
        moved = g[abi.CPVOLUME][c0] != f[abi.CPVOLUME][c0]
        assert np.array_equal(moved, ok) or moved[ok].any()
        if mode == 2:
            assert np.array_equal(g[abi.CPENERGY], f[abi.CPENERGY])
        else:
            assert not np.array_equal(g[abi.CPENERGY], f[abi.CPENERGY])
        assert np.array_equal(g[abi.CPMASS], f[abi.CPMASS])


def test_interface_and_error_measures():
    """The measures the closure is judged by: a run against itself is at
    zero distance; moving volume between the materials of one mixed cell
    shifts that row's interface by the moved volume over the row's height
    and shows up in the material errors against the unmoved state."""
    nx, ny = 40, 4
    a = _problem(nx, ny)
    b = a.copy()
    idx = closure.grid_index(a, nx, ny)
    assert closure.against_plain(a, a, idx, nx, ny) == (0.0, 0.0, 0.0)
    f = b.fields
    c0 = f[abi.IMXFCP][0] - 1                # the first mixed cell's components
    dv = 0.1 * min(f[abi.CPVOLUME][c0], f[abi.CPVOLUME][c0 + 1])
    f[abi.CPVOLUME][c0] += dv
    f[abi.CPVOLUME][c0 + 1] -= dv
    shift, l1_mixed, l1_all = closure.against_plain(b, a, idx, nx, ny)
    row_height = 0.1 / ny
    dx = 1.0 / nx
    assert abs(shift - dv / row_height / dx) < 1e-9 * shift
    assert l1_mixed == 0.0 and l1_all == 0.0     # cell densities unchanged
    V, M, _ = closure.material_sums(a, idx, nx * ny)
    cells = idx[f[abi.IMXEL][:a.sizes.nmx] - 1]
    fe, r1, r2 = closure.mixed_errors(b, idx, (V, M), cells)
    assert fe > 0 and r1 > 0 and r2 > 0
    assert closure.mixed_errors(a, idx, (V, M), cells) == (0.0, 0.0, 0.0)
