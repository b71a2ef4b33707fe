"""bl_getdt_noalloc: the allocation-free getdt for callers that cannot call
cudaMalloc (a host that owns all device memory in its own pool and hands it
out itself).  It runs the library's exact-form k_getdt on arrays in the
reference's layout, so it is checked, through the C-ABI, bit for bit
against the existing entry point bl_getdt in exact mode and against the
CPU restatement on the same state, on two calls in a row (the second call
reuses the fixed scratch array the first one left behind): a single-region
Sedov mesh, a 64x64 two-region mesh with zdtnotreg and zmidlength set, and
a deck with the tensor viscosity switch (ztq, viscosity taken as given).

This file is named so that pytest collects it last.
"""
import ctypes as ct

import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, Solver, abi, configs

pytestmark = pytest.mark.gpu


class GetdtArrays(ct.Structure):
    """Mirror of bl_getdt_arrays (include/bookleaf_gb300.h)."""
    _fields_ = [("nel", ct.c_int), ("nnd", ct.c_int)] + [
        (n, ct.c_void_p) for n in (
            "ndx", "ndy", "ndu", "ndv", "indtype", "ielnd", "ielel", "ielfc", "ielreg",
            "eldensity", "elcs2", "a1", "a3", "b1", "b3", "elvolume", "cnviscx", "cnviscy",
            "elvisc", "elcs2_out")]


def _state_after(deck, steps):
    p = Problem.from_deck(deck)
    s = Solver(p, fp_mode=abi.FP_EXACT)
    for _ in range(steps):
        assert s.step() == 0, s.error.message
    s.sync_to_host(0)
    s.close()
    return p


TWO_REGION = configs.sod(64, 64).replace(
    "cvisc2=0.75\n", "cvisc2=0.75\n zmidlength(2)=.TRUE.\n zdtnotreg(1)=.TRUE.\n")
TENSOR = configs.sod(64, 16).replace("cvisc2=0.75\n", "cvisc2=0.75\n visc='TENSOR'\n")
CASES = {"sedov_24": (configs.sedov(24), 4), "sod_64x64_two_regions": (TWO_REGION, 6),
         "sod_64x16_tensor": (TENSOR, 3)}


@pytest.mark.parametrize("name", list(CASES))
def test_noalloc_matches_getdt_and_oracle_twice(name):
    import torch
    from bookleaf_f90_gb300 import _lib
    from oracle.oracle import Oracle
    L = _lib.load()
    L.bl_getdt_noalloc.argtypes = [ct.POINTER(GetdtArrays), ct.POINTER(abi.Config),
                                   ct.POINTER(abi.Timestep), ct.c_void_p, ct.POINTER(abi.Error)]
    L.bl_getdt_noalloc.restype = ct.c_int
    torch.cuda.init()

    deck, steps = CASES[name]
    p = _state_after(deck, steps)
    if name == "sod_64x64_two_regions":
        assert p.sizes.nreg == 2 and p.config.zdtnotreg[0] and p.config.zmidlength[1]
    if name == "sod_64x16_tensor":
        assert p.config.ztq
    # the existing entry point (exact mode) and the CPU restatement on the
    # same state
    q = p.copy()
    sref = Solver(q, fp_mode=abi.FP_EXACT)
    ts_ref = q.timestep.copy()
    assert sref.inf_solver_getdt(ts_ref) == 0, sref.error.message
    sref.sync_to_host(0)
    sref.close()
    o_p = p.copy()
    ts_orc = o_p.timestep.copy()
    orc = Oracle(o_p)
    assert orc.getdt(ts_orc) == 0

    dev = torch.device("cuda:0")
    keep = []

    def d(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        keep.append(t)
        return t.data_ptr()

    f = p.fields
    outs = {k: torch.zeros(f[k].shape, dtype=torch.float64, device=dev)
            for k in (abi.CNVISCX, abi.CNVISCY)}
    # the tensor switch takes elvisc as given: pass it in
    outs[abi.ELVISC] = torch.from_numpy(f[abi.ELVISC].copy()).to(dev)
    cs2_out = torch.zeros(f[abi.ELCS2].shape, dtype=torch.float64, device=dev)
    A = GetdtArrays()
    A.nel, A.nnd = p.nel, p.nnd
    for nm, fid in (("ndx", abi.NDX), ("ndy", abi.NDY), ("ndu", abi.NDU), ("ndv", abi.NDV),
                    ("indtype", abi.INDTYPE), ("ielnd", abi.IELND), ("ielel", abi.IELEL),
                    ("ielfc", abi.IELFC), ("ielreg", abi.IELREG), ("eldensity", abi.ELDENSITY),
                    ("elcs2", abi.ELCS2), ("a1", abi.A1), ("a3", abi.A3), ("b1", abi.B1),
                    ("b3", abi.B3), ("elvolume", abi.ELVOLUME)):
        setattr(A, nm, d(f[fid]))
    A.cnviscx = outs[abi.CNVISCX].data_ptr()
    A.cnviscy = outs[abi.CNVISCY].data_ptr()
    A.elvisc = outs[abi.ELVISC].data_ptr()
    A.elcs2_out = cs2_out.data_ptr()
    torch.cuda.synchronize()

    for call in range(2):
        ts = p.timestep.copy()
        err = abi.Error()
        ierr = L.bl_getdt_noalloc(ct.byref(A), ct.byref(p.config), ct.byref(ts), None,
                                  ct.byref(err))
        assert ierr == 0, err.message
        for ref in (ts_ref, ts_orc):
            assert (ts.nstep, ts.idtel, ts.sdt, ts.dt, ts.time) == (
                ref.nstep, ref.idtel, ref.sdt, ref.dt, ref.time), (call, ts.as_tuple())
        for fid, t in outs.items():
            got = t.cpu().numpy()
            assert np.array_equal(got, q.fields[fid]), (call, abi.NAMES[fid])
            assert np.array_equal(got, o_p.fields[fid]), (call, abi.NAMES[fid])
        got = cs2_out.cpu().numpy()
        # elcs2 + elvisc: bl_getdt and the restatement hold it in elcs2
        assert np.array_equal(got, q.fields[abi.ELCS2]), call
        assert np.array_equal(got, o_p.fields[abi.ELCS2]), call
        # clear the outputs so the second call has to write them again
        # (elvisc is an input under the tensor switch)
        outs[abi.CNVISCX].zero_()
        outs[abi.CNVISCY].zero_()
        if not p.config.ztq:
            outs[abi.ELVISC].zero_()
        cs2_out.zero_()
        torch.cuda.synchronize()


def test_noalloc_rejects_aliased_cs2():
    from bookleaf_f90_gb300 import _lib
    L = _lib.load()
    L.bl_getdt_noalloc.argtypes = [ct.POINTER(GetdtArrays), ct.POINTER(abi.Config),
                                   ct.POINTER(abi.Timestep), ct.c_void_p, ct.POINTER(abi.Error)]
    L.bl_getdt_noalloc.restype = ct.c_int
    A = GetdtArrays()
    A.nel, A.nnd = 16, 25
    for nm, _ in GetdtArrays._fields_[2:]:
        setattr(A, nm, 4096)            # never dereferenced: rejected first
    A.elcs2_out = A.elcs2
    err = abi.Error()
    ts = abi.Timestep()
    cfg = abi.Config()
    assert L.bl_getdt_noalloc(ct.byref(A), ct.byref(cfg), ct.byref(ts), None,
                              ct.byref(err)) == abi.FAILURE
    assert "alias" in err.message


def test_noalloc_rejects_oversized_mesh():
    from bookleaf_f90_gb300 import _lib
    L = _lib.load()
    L.bl_getdt_noalloc.argtypes = [ct.POINTER(GetdtArrays), ct.POINTER(abi.Config),
                                   ct.POINTER(abi.Timestep), ct.c_void_p, ct.POINTER(abi.Error)]
    L.bl_getdt_noalloc.restype = ct.c_int
    A = GetdtArrays()
    A.nel, A.nnd = 65536 * 128 + 1, 10
    err = abi.Error()
    ts = abi.Timestep()
    cfg = abi.Config()
    assert L.bl_getdt_noalloc(ct.byref(A), ct.byref(cfg), ct.byref(ts), None,
                              ct.byref(err)) == abi.FAILURE
    assert "BL_NOALLOC_MAX_NEL" in err.message
