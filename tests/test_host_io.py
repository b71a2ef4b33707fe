"""The driver's visualisation dump (bookleaf_gb300 --vtk-setup, io.cpp),
the reference's Silo dump (io_dr_silo.f90:70-262) as a VTK legacy
unstructured grid: mesh, element variables, region, materials with their
volume fractions, node velocity -- checked value for value against the
Python set-up of the same control file.  CPU only (the set-up dump touches
no GPU)."""
import subprocess

import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, abi, configs
from bookleaf_f90_gb300 import build as blbuild
from vtk_read import read_vtk

import golden


@pytest.fixture(scope="module")
def exe():
    blbuild.build()
    return blbuild.EXE


@pytest.mark.parametrize("name", ["sod_multimaterial", "noh_small", "sod_mm_lag_small"])
def test_vtk_dump_of_the_initial_state(exe, tmp_path, name):
    deck = (configs.sod_multimaterial(20, 4) if name == "sod_multimaterial"
            else golden.deck_text(name))
    dpath = tmp_path / "deck"
    dpath.write_text(deck)
    out = tmp_path / "dump.vtk"
    r = subprocess.run([exe, "--vtk-setup", str(out), str(dpath)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    title, pts, cells, cd, pd = read_vtk(out)
    p = Problem.from_deck(deck)
    f = p.fields
    assert "nstep=0" in title
    assert np.array_equal(pts[:, 0], f[abi.NDX]) and np.array_equal(pts[:, 1], f[abi.NDY])
    assert np.array_equal(cells, f[abi.IELND].reshape(-1, 4) - 1)
    for nm, fid in (("density", abi.ELDENSITY), ("energy", abi.ELENERGY),
                    ("pressure", abi.ELPRESSURE), ("region", abi.IELREG),
                    ("material", abi.IELMAT)):
        assert np.array_equal(cd[nm], f[fid]), nm
    assert np.array_equal(pd["velocity"][:, 0], f[abi.NDU])
    assert np.array_equal(pd["velocity"][:, 1], f[abi.NDV])
    vf = np.array([v for k, v in cd.items() if k.startswith("volume_fraction_")])
    assert vf.shape[0] == p.sizes.nmat
    assert np.allclose(vf.sum(axis=0), 1.0, rtol=0, atol=1e-15)
    mixed = f[abi.IELMAT] <= 0
    assert mixed.sum() == p.sizes.nmx
    if p.sizes.nmx:
        assert np.all((vf[:, mixed] > 0).sum(axis=0) >= 2)
