"""The C++ driver (bookleaf_gb300) runs control files end to end on the GPU
through the C++ host side: set-up, solver entry points (per call, or the
device loop), short print and Sod validation.  Its final state must equal
the Python-hosted path's bit for bit in exact mode."""
import os
import re
import subprocess

import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, Solver, abi, configs
from bookleaf_f90_gb300 import build as blbuild
from test_host_setup import read_dump

pytestmark = pytest.mark.gpu


def _python_final(deck, exact=True):
    p = Problem.from_deck(deck)
    s = Solver(p, fp_mode=abi.FP_EXACT if exact else abi.FP_FAST)
    ierr, _ = s.run(history=False)
    assert ierr == 0, s.error.message
    s.sync_to_host(0)
    return p


def _driver(tmp_path, deck, name, *args):
    blbuild.build()
    d = tmp_path / name
    d.write_text(deck)
    out = tmp_path / (name + ".final")
    r = subprocess.run([blbuild.EXE, "--dump-final", str(out)] + list(args) + [str(d)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout, read_dump(out)


@pytest.mark.parametrize("mode", [[], ["--calls"]])
def test_driver_matches_python_path_exact(tmp_path, mode):
    deck = configs.sedov(24, time_end=0.05, kappa=0.01, pmerit=0.1)
    out, (sizes, config, ts, fields) = _driver(tmp_path, deck, "sedov_deck", "--fp", "exact", *mode)
    p = _python_final(deck)
    assert ts.nstep == p.timestep.nstep and ts.time == p.timestep.time
    for fid in (abi.ELDENSITY, abi.ELENERGY, abi.ELPRESSURE, abi.ELVOLUME, abi.NDX, abi.NDY,
                abi.NDU, abi.NDV, abi.CNMASS, abi.CNVISCX):
        assert np.array_equal(fields[fid], np.ascontiguousarray(p.fields[fid]).reshape(-1)), abi.NAMES[fid]
    assert "Step no." in out and "total energy" in out


def test_driver_sod_validation(tmp_path):
    """The Sod check of the driver (check_kn_sod restated in C++) on the
    reference check's geometry agrees with the CPU restatement's."""
    from oracle.oracle import sod_l1
    deck = configs.sod_reference(100, 5)
    out, (sizes, config, ts, fields) = _driver(tmp_path, deck, "sod_ref_deck", "--fp", "exact")
    m = re.search(r"L1 norm\. of density:\s+(\S+)", out)
    assert m, out[-1000:]
    l1 = float(m.group(1))
    p = _python_final(deck)
    ref = sod_l1(p, p.timestep.time)[0]
    assert abs(l1 - ref) <= 1e-9 * abs(ref), (l1, ref)
    assert 1e-3 < l1 < 2e-2


def test_driver_vtk_dump_of_the_final_state(tmp_path):
    """--vtk writes the reference's visualisation dump (as VTK) of the
    state at the end of the run: the mesh and fields equal the Python path's
    final state bit for bit in exact mode, mixed cells included."""
    from vtk_read import read_vtk
    deck = configs.sod_multimaterial(40, 6, time_end=2.0)
    vtk = tmp_path / "final.vtk"
    out, (sizes, config, ts, fields) = _driver(tmp_path, deck, "sod_mm_deck", "--fp", "exact",
                                               "--vtk", str(vtk))
    title, pts, cells, cd, pd = read_vtk(vtk)
    p = _python_final(deck)
    assert "nstep=%d" % p.timestep.nstep in title
    assert np.array_equal(pts[:, 0], p.fields[abi.NDX])
    assert np.array_equal(pts[:, 1], p.fields[abi.NDY])
    assert np.array_equal(cd["density"], p.fields[abi.ELDENSITY])
    assert np.array_equal(cd["pressure"], p.fields[abi.ELPRESSURE])
    assert np.array_equal(pd["velocity"][:, 0], p.fields[abi.NDU])
    vf = np.array([v for k, v in cd.items() if k.startswith("volume_fraction_")])
    assert np.allclose(vf.sum(axis=0), 1.0, rtol=0, atol=1e-12)
