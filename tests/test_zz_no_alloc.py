"""bl_getdt_noalloc: the allocation-free getdt for callers that cannot call
cudaMalloc (a host that owns all device memory in its own pool, or work that
must not allocate).  It is checked, through the C-ABI, against the existing
entry point bl_getdt on the same state, on two calls in a row (the second
call reuses the fixed scratch array the first one left behind).

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
    s = Solver(p, fp_mode=abi.FP_FAST)
    for _ in range(steps):
        assert s.step() == 0, s.error.message
    s.sync_to_host(0)
    s.close()
    return p


def test_noalloc_matches_getdt_twice():
    import torch
    from bookleaf_f90_gb300 import _lib
    L = _lib.load()
    L.bl_getdt_noalloc.argtypes = [ct.POINTER(GetdtArrays), ct.POINTER(abi.Config),
                                   ct.POINTER(abi.Timestep), ct.c_void_p, ct.POINTER(abi.Error)]
    L.bl_getdt_noalloc.restype = ct.c_int
    torch.cuda.init()

    p = _state_after(configs.sedov(24), 4)
    # the existing entry point on the same state
    q = p.copy()
    sref = Solver(q, fp_mode=abi.FP_FAST)
    ts_ref = q.timestep.copy()
    assert sref.inf_solver_getdt(ts_ref) == 0, sref.error.message
    sref.sync_to_host(0)
    sref.close()

    dev = torch.device("cuda:0")
    keep = []

    def d(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        keep.append(t)
        return t.data_ptr()

    f = p.fields
    outs = {k: torch.zeros(f[k].shape, dtype=torch.float64, device=dev)
            for k in (abi.CNVISCX, abi.CNVISCY, abi.ELVISC)}
    cs2_out = torch.zeros(f[abi.ELCS2].shape, dtype=torch.float64, device=dev)
    A = GetdtArrays()
    A.nel, A.nnd = p.nel, p.nnd
    for name, fid in (("ndx", abi.NDX), ("ndy", abi.NDY), ("ndu", abi.NDU), ("ndv", abi.NDV),
                      ("indtype", abi.INDTYPE), ("ielnd", abi.IELND), ("ielel", abi.IELEL),
                      ("ielfc", abi.IELFC), ("ielreg", abi.IELREG), ("eldensity", abi.ELDENSITY),
                      ("elcs2", abi.ELCS2), ("a1", abi.A1), ("a3", abi.A3), ("b1", abi.B1),
                      ("b3", abi.B3), ("elvolume", abi.ELVOLUME)):
        setattr(A, name, d(f[fid]))
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
        assert (ts.nstep, ts.idtel, ts.sdt) == (ts_ref.nstep, ts_ref.idtel, ts_ref.sdt), call
        assert ts.dt == pytest.approx(ts_ref.dt, rel=1e-11)
        assert ts.time == pytest.approx(ts_ref.time, rel=1e-11)
        for fid, t in outs.items():
            np.testing.assert_allclose(t.cpu().numpy(), q.fields[fid], rtol=1e-11, atol=1e-14)
        np.testing.assert_allclose(cs2_out.cpu().numpy(), q.fields[abi.ELCS2], rtol=1e-11,
                                   atol=1e-14)
        # clear the outputs so the second call has to write them again
        for t in outs.values():
            t.zero_()
        cs2_out.zero_()
        torch.cuda.synchronize()


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
