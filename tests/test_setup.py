"""Host-side set-up: control-file reader, mesh, connectivity, node types,
initial conditions (CPU only)."""
import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, abi, configs
from bookleaf_f90_gb300.setup import deck, mesh


def test_namelist_sections_and_lists():
    g = deck.parse("""&MESH
 region_dim(1,:)=400,40
 segment_typ(:)='LINE','LINE','LINE','LINE'
 segment_pos(2,:)=1.0,0.0,1.0,0.1
/
&INITIAL_CONDITIONS
 kinematic_param(1,1)=-1.0
 kinematic_param(2:3,1)=0.0
 density(2)=0.125   ! comment
/
""")
    m = g["mesh"]
    assert m["region_dim"][(1, 1)] == 400 and m["region_dim"][(1, 2)] == 40
    assert [m["segment_typ"][(i,)] for i in range(1, 5)] == ["LINE"] * 4
    assert m["segment_pos"][(2, 4)] == 0.1
    ic = g["initial_conditions"]
    assert ic["kinematic_param"][(2, 1)] == 0.0
    assert (3, 1) not in ic["kinematic_param"]  # one value fills one element
    assert ic["density"][(2,)] == 0.125


def test_lin1_numbering_matches_reference_layout():
    p = Problem.from_deck(configs.sod(8, 3))
    nd = p.fields[abi.IELND]
    # l (region_dim(:,2)) runs fastest: element 1 is the lower-left cell,
    # corners counter-clockwise (setup_mesh.F90:1216-1225)
    assert list(nd[0]) == [1, 5, 6, 2]
    assert list(nd[1]) == [2, 6, 7, 3]
    x, y = p.fields[abi.NDX], p.fields[abi.NDY]
    # the corner is written last by side 4 (0.1 + 3*(-0.1)/3): -1.4e-17, as
    # setup_mesh_line's arithmetic gives in the reference
    assert x[0] == 0.0 and abs(y[0]) < 1e-16
    assert y[3] == pytest.approx(0.1) and x[4] == pytest.approx(1 / 8)
    assert np.all(p.fields[abi.ELVOLUME] > 0)
    assert p.fields[abi.ELVOLUME].sum() == pytest.approx(0.1)


def test_connectivity_is_symmetric():
    p = Problem.from_deck(configs.sedov(7))
    el, fc = p.fields[abi.IELEL], p.fields[abi.IELFC]
    nel = p.nel
    for iel in range(nel):
        for j in range(4):
            nb, f = el[iel, j] - 1, fc[iel, j] - 1
            if nb == iel:
                assert f == (j + 2) % 4    # boundary: self, opposite face
            else:
                assert el[nb, f] - 1 == iel and fc[nb, f] - 1 == j


def test_node_types_and_corner_bc():
    p = Problem.from_deck(configs.sod(6, 3))
    t = p.fields[abi.INDTYPE]
    # corners between a SLIPX and a SLIPY side become WALL (-3)
    no_l = 4
    corners = [0, no_l - 1, 6 * no_l, 7 * no_l - 1]
    assert all(t[c] == -3 for c in corners)
    assert np.all(t[[1, 2]] == -1)          # left edge SLIPX
    assert t[no_l] == -2                    # bottom edge SLIPY
    assert t[no_l + 1] == 1                 # interior: mesh region 1


def test_sod_initial_state():
    p = Problem.from_deck(configs.sod(10, 2))
    rho, e = p.fields[abi.ELDENSITY], p.fields[abi.ELENERGY]
    assert set(np.unique(rho)) == {1.0, 0.125}
    assert np.all(p.fields[abi.ELPRESSURE][rho == 1.0] == pytest.approx(1.0))
    assert np.all(p.fields[abi.ELPRESSURE][rho == 0.125] == pytest.approx(0.1))
    assert p.config.zhg == 0 and p.config.zsp == 0


def test_sedov_energy_deposit_and_noh_velocity():
    p = Problem.from_deck(configs.sedov(16))
    e, v = p.fields[abi.ELENERGY], p.fields[abi.ELVOLUME]
    assert e[0] * v[0] == pytest.approx(0.244816)
    assert e[1] == 1.0e-12
    q = Problem.from_deck(configs.noh(8))
    u, w = q.fields[abi.NDU], q.fields[abi.NDV]
    assert u[0] == 0.0 and w[0] == 0.0           # origin, WALL corner
    r = np.hypot(q.fields[abi.NDX], q.fields[abi.NDY])
    inner = (q.fields[abi.INDTYPE] > 0)
    assert np.allclose(np.hypot(u, w)[inner], 1.0)
    assert np.all(u[inner] * q.fields[abi.NDX][inner] <= 0)
    assert r.max() == pytest.approx(np.sqrt(2))


def test_multimaterial_components():
    p = Problem.from_deck(configs.sod_multimaterial(20, 4))
    s = p.sizes
    assert s.nmx == 4 and s.ncp == 8               # one column of mixed cells
    assert np.all(p.fields[abi.IELMAT][p.fields[abi.IMXEL] - 1] < 0)
    fr = p.fields[abi.FRVOLUME]
    assert np.allclose(fr, 0.5)
    assert list(p.fields[abi.ICPMAT][:2]) == [1, 2]


def test_reference_decks_parse():
    """Every control file of the reference (vendored under
    tests/golden/decks) sets up a mesh of positive volumes; the two
    14M-element decks are the medium ones refined and are set up by the
    C++/Python equality test instead."""
    import golden
    for d in golden.deck_names():
        if d.startswith("sod_sm_") and d.endswith("_large"):
            continue
        p = Problem.from_deck(golden.deck_text(d))
        assert p.nel > 0 and np.all(p.fields[abi.ELVOLUME] > 0), d


def test_noh_decks_polar_mesh():
    """The reference's Noh decks (input/noh_small, noh_large) have curved
    sides (ARC_A outer radius 1, ARC_C inner radius 0.005, both centred on
    the origin): every node on them lies at its radius, the side nodes are
    equally spaced in angle, the mesh fills the quarter annulus up to the
    chords' sagitta, and the initial velocity is unit and radial inwards."""
    import golden
    p = Problem.from_deck(golden.deck_text("noh_small"))
    x, y = p.fields[abi.NDX], p.fields[abi.NDY]
    r = np.hypot(x, y)
    no_l, no_k = 31, 76                       # region_dim(1,:) = 75,30
    rr = r.reshape(no_k, no_l)
    assert np.allclose(rr[-1, :], 1.0, rtol=0, atol=1e-15)
    assert np.allclose(rr[0, :], 0.005, rtol=0, atol=1e-17)
    th = np.arctan2(y, x).reshape(no_k, no_l)
    dth = np.diff(th[-1, :])
    assert np.allclose(dth, dth[0], rtol=1e-12) and abs(abs(dth.sum()) - np.pi / 2) < 1e-14
    area = np.pi / 4 * (1 - 0.005 ** 2)
    sag = 1 - np.cos(np.pi / 4 / 30)          # chord sagitta loss per unit radius^2
    assert 0 < area - p.fields[abi.ELVOLUME].sum() < 2 * sag * area
    u, v = p.fields[abi.NDU], p.fields[abi.NDV]
    it = p.fields[abi.INDTYPE]
    free = it > 0
    assert np.allclose(np.hypot(u, v)[free], 1.0, atol=1e-15)
    assert np.allclose((u * x + v * y)[free] / r[free], -1.0, atol=1e-15)
    # the inner arc is a WALL (-3): the boundary condition zeroes its velocity
    assert np.all(it.reshape(no_k, no_l)[0, :] == -3)
    assert np.all((u == 0) & (v == 0) | (it != -3))


def test_sinusoidal_interface_fractions_are_exact_areas():
    """The two-material Sod's cell fractions of material 2 add up to its
    area (half the tube: the sine integrates to zero over whole periods),
    and the mixed cells straddle the interface."""
    import numpy as np
    from bookleaf_f90_gb300 import Problem, abi, configs
    deck, frac = configs.sod_interface(200, 20, time_end=0.01)
    p = Problem.from_deck(deck, material_fraction=frac)
    nd = p.fields[abi.IELND].reshape(-1, 4) - 1
    cnx, cny = p.fields[abi.NDX][nd], p.fields[abi.NDY][nd]
    vf = frac(cnx, cny)
    area = p.fields[abi.ELVOLUME]
    assert abs(np.sum(vf * area) - 0.05) <= 1e-9
    assert p.sizes.nmx == int(np.sum((vf > 0) & (vf < 1))) > 20
    assert p.sizes.ncp == 2 * p.sizes.nmx


def test_noh_polar_generator_is_the_reference_deck():
    """configs.noh_polar(75, 30), the generator of the Noh benchmark on the
    reference's polar mesh, sets up the reference's own input/noh_small
    exactly (every field and the configuration)."""
    import golden
    a = Problem.from_deck(configs.noh_polar(75, 30))
    b = Problem.from_deck(golden.deck_text("noh_small"))
    assert bytes(a.config) == bytes(b.config)
    assert set(a.fields) == set(b.fields)
    for fid in b.fields:
        assert np.array_equal(a.fields[fid], b.fields[fid]), abi.NAMES[fid]
