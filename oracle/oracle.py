"""ctypes wrapper of the CPU restatement (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg.  Never used by the product.
Parity status: pinned by the reference's Sod known-answer test and by
conservation invariants only (see oracle.h).
"""
import ctypes as ct
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = [os.path.join(HERE, "oracle.c")]
HDR = [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "..", "include", "bookleaf_gb300.h")]

# -ffp-contract=off: gcc contracts a*b+c into fma by default on aarch64.
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11"]


def build(force=False):
    """Compile oracle.c into oracle/_build/liboracle.so."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SRC + HDR)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc"] + CFLAGS + SRC + ["-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        import sys
        sys.path.insert(0, os.path.join(HERE, ".."))
        from bookleaf_f90_gb300 import abi
        L = ct.CDLL(build())
        P = ct.POINTER
        L.orc_init.restype = ct.c_void_p
        L.orc_init.argtypes = [P(abi.Sizes), P(abi.Config), ct.c_void_p, P(abi.Error)]
        L.orc_finalize.argtypes = [ct.c_void_p]
        for nm in ("orc_getdt", "orc_lagstep"):
            getattr(L, nm).argtypes = [ct.c_void_p, P(abi.Timestep), P(abi.Error)]
            getattr(L, nm).restype = ct.c_int
        L.orc_alestep.argtypes = [ct.c_void_p, P(abi.Timestep), P(abi.Error)]
        L.orc_alestep.restype = ct.c_int
        L.orc_field.argtypes = [ct.c_void_p, ct.c_int]
        L.orc_field.restype = ct.c_void_p
        L.orc_sod_l1.argtypes = [ct.c_int, ct.c_double] + [ct.c_void_p] * 5 + [ct.c_void_p]
        _lib = L
    return _lib


class Oracle:
    """The reference's three solver entry points on the CPU, in place on a
    Problem's host arrays (like the Fortran host's dh(:))."""

    def __init__(self, problem):
        from bookleaf_f90_gb300 import abi
        self.abi = abi
        self.p = problem
        self.L = lib()
        self.err = abi.Error()
        self._tab = problem.pointer_table()
        self.ctx = self.L.orc_init(ct.byref(problem.sizes), ct.byref(problem.config),
                                   ct.cast(self._tab, ct.c_void_p), ct.byref(self.err))

    def __del__(self):
        try:
            if self.ctx:
                self.L.orc_finalize(self.ctx)
                self.ctx = None
        except Exception:
            pass

    def getdt(self, ts):
        return self.L.orc_getdt(self.ctx, ct.byref(ts), ct.byref(self.err))

    def lagstep(self, ts):
        return self.L.orc_lagstep(self.ctx, ct.byref(ts), ct.byref(self.err))

    def alestep(self, ts):
        return self.L.orc_alestep(self.ctx, ct.byref(ts), ct.byref(self.err))

    def step(self, ts):
        """One cycle of inf_control_solver's loop (getdt, lagstep, alestep)."""
        for fn in (self.getdt, self.lagstep, self.alestep):
            ierr = fn(ts)
            if ierr != 0:
                return ierr
        return 0

    def run(self, ts, max_steps=10**9):
        """Time loop until time >= time_end (time_finish) or an error."""
        n = 0
        while n < max_steps:
            ierr = self.step(ts)
            n += 1
            if ierr != 0:
                return ierr, n
            if ts.time >= self.p.config.time_end:
                break
        return 0, n

    def scratch(self, fid, n, dtype="f8"):
        import numpy as np
        ptr = self.L.orc_field(self.ctx, fid)
        return np.ctypeslib.as_array(ct.cast(ptr, ct.POINTER(ct.c_double if dtype == "f8" else ct.c_int)),
                                     shape=(n,)).copy()


def sod_l1(problem, time):
    """check_dr_sod: (density L1, energy L1) vs the exact solution."""
    import numpy as np
    from bookleaf_f90_gb300 import abi
    f = problem.fields
    nd = f[abi.IELND] - 1
    cnx = np.ascontiguousarray(f[abi.NDX][nd])
    cny = np.ascontiguousarray(f[abi.NDY][nd])
    out = (ct.c_double * 2)()
    lib().orc_sod_l1(problem.nel, time, f[abi.ELVOLUME].ctypes.data, f[abi.ELDENSITY].ctypes.data,
                     f[abi.ELENERGY].ctypes.data, cnx.ctypes.data, cny.ctypes.data,
                     ct.cast(out, ct.c_void_p))
    return out[0], out[1]
