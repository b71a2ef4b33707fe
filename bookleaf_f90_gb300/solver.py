"""Host-side mirror of the reference's solver interface for the hot path.

``Solver`` is the Python counterpart of a Fortran host that calls the
C-ABI: it registers a Problem's host arrays (like the reference's dh(:)),
and exposes the three entry points under the reference's names

    inf_solver_getdt   (src/infrastructure/solver/inf_solver_getdt.f90:35-70)
    inf_solver_lagstep (src/infrastructure/solver/inf_solver_lagstep.f90:44-78)
    inf_solver_alestep (src/infrastructure/solver/inf_solver_alestep.f90:39-74)

with the reference's error behaviour: each returns error%ierr, and a
non-zero return carries error%iout/serr in ``Solver.error`` (the Fortran
wrapper would then call inf_error_halt).  ``run`` is the time loop of
inf_control_solver (inf_control_solver.f90:53-69) executed on the device.
"""
import ctypes as ct

import numpy as np

from . import abi
from ._lib import load


class SolverError(RuntimeError):
    def __init__(self, ierr, iout, message):
        super().__init__("%s (ierr=%d, iout=%d)" % (message, ierr, iout))
        self.ierr = ierr
        self.iout = iout
        self.message = message


class Solver:
    def __init__(self, problem, fp_mode=abi.FP_FAST):
        self.L = load()
        self.problem = problem
        self.timestep = problem.timestep
        self.error = abi.Error()
        self._tab = problem.pointer_table()
        self.ctx = ct.c_void_p()
        ierr = self.L.bl_init(ct.byref(self.ctx), ct.byref(problem.sizes),
                              ct.byref(problem.config), ct.cast(self._tab, ct.c_void_p),
                              int(fp_mode), ct.byref(self.error))
        if ierr != 0:
            raise SolverError(ierr, self.error.iout, self.error.message)

    # ---- the reference's entry points -------------------------------------
    def inf_solver_getdt(self, ts=None):
        return self.L.bl_getdt(self.ctx, ct.byref(ts or self.timestep), ct.byref(self.error))

    def inf_solver_lagstep(self, ts=None):
        return self.L.bl_lagstep(self.ctx, ct.byref(ts or self.timestep), ct.byref(self.error))

    def inf_solver_alestep(self, ts=None):
        return self.L.bl_alestep(self.ctx, ct.byref(ts or self.timestep), ct.byref(self.error))

    def step(self, ts=None):
        """One cycle of inf_control_solver's loop; returns error%ierr."""
        ts = ts or self.timestep
        for fn in (self.inf_solver_getdt, self.inf_solver_lagstep, self.inf_solver_alestep):
            ierr = fn(ts)
            if ierr != 0:
                return ierr
        return 0

    def run(self, max_steps=10**9, ts=None, history=True):
        """Device-resident time loop until time_end, max_steps or an error.
        Returns (ierr, list of (nstep, time, dt, idtel, sdt))."""
        ts = ts or self.timestep
        max_steps = int(min(max_steps, 2**31 - 1))
        hist = (abi.StepRecord * max_steps)() if history else None
        n = ct.c_int(0)
        ierr = self.L.bl_run(self.ctx, ct.byref(ts), max_steps,
                             ct.cast(hist, ct.c_void_p) if history else None, ct.byref(n),
                             ct.byref(self.error))
        recs = []
        if history:
            for i in range(n.value):
                r = hist[i]
                recs.append((r.nstep, r.time, r.dt, r.idtel, abi.DT_NAMES[r.sdt_code]))
        return ierr, recs

    # ---- diagnostics on the device -------------------------------------------
    SHORTPRINT_COLUMNS = ("vol", "mass", "ie", "ke", "pressure", "pmn", "pmx", "density",
                          "dmn", "dmx")

    def shortprint(self, by_material=False):
        """hydro_dr_shortprint's per-region (or per-material) table from the
        device state: a list of dicts with SHORTPRINT_COLUMNS."""
        n = self.problem.sizes.nmat if by_material else self.problem.sizes.nreg
        out = (ct.c_double * (n * 10))()
        if self.L.bl_shortprint(self.ctx, int(by_material), out, n, ct.byref(self.error)) != 0:
            raise SolverError(-1, self.error.iout, self.error.message)
        return [dict(zip(self.SHORTPRINT_COLUMNS, out[10 * i:10 * i + 10])) for i in range(n)]

    def check_sod(self, time=None):
        """check_dr_sod on the device: (density L1, energy L1)."""
        t = self.timestep.time if time is None else time
        d, e = ct.c_double(), ct.c_double()
        if self.L.bl_check_sod(self.ctx, t, ct.byref(d), ct.byref(e), ct.byref(self.error)) != 0:
            raise SolverError(-1, self.error.iout, self.error.message)
        return d.value, e.value

    # ---- data movement ------------------------------------------------------
    def sync_to_host(self, fid=0):
        if self.L.bl_sync_to_host(self.ctx, int(fid)) != 0:
            raise RuntimeError("bl_sync_to_host failed")

    def sync_to_device(self, fid=0):
        if self.L.bl_sync_to_device(self.ctx, int(fid)) != 0:
            raise RuntimeError("bl_sync_to_device failed")

    def synchronize(self):
        return self.L.bl_synchronize(self.ctx)

    @property
    def stream(self):
        return self.L.bl_stream(self.ctx)

    def time_step_kernels(self, nstep=16, ts=None):
        """Advances nstep Lagrangian steps with the four kernels queued back
        to back and CUDA events between them; returns (ierr, [ms of getdt,
        lag_force, lag_accel, lag_state], each the mean over the steps)."""
        ts = ts or self.timestep
        ms = (ct.c_double * 4)()
        ierr = self.L.bl_time_step_kernels(self.ctx, ct.byref(ts), int(nstep), ms, 4,
                                           ct.byref(self.error))
        return ierr, list(ms)

    # ---- the learned mixed-cell closure -------------------------------------
    def set_closure(self, net, norm, on=True, volume_only=False):
        """Let the network net (closure.ClosureNet; its current parameters
        are copied) split each two-material cell's volume change between its
        materials from the next Lagrangian step on, with the feature
        standardisation norm (22 floats, see closure.fit_norm); on=False
        restores the plain closure.  By default the moved volume trades
        energy at the mixture pressure; with volume_only the materials keep
        their specific energies and, for ideal gases, the flow stays the
        plain closure's (only the split between the materials changes)."""
        nm_arr = np.ascontiguousarray(norm, dtype=np.float32) if on else None
        if on and nm_arr.size != 22:
            raise ValueError("norm needs 22 floats")
        nm = nm_arr.ctypes.data_as(ct.c_void_p) if on else None
        mode = (2 if volume_only else 1) if on else 0
        if self.L.bl_set_closure(self.ctx, net.handle if on else None, nm, mode,
                                 ct.byref(self.error)) != 0:
            raise SolverError(-1, self.error.iout, self.error.message)

    def closure_stats(self):
        """(mixed-cell steps the closure saw, those it left to the plain
        closure)."""
        a, b = ct.c_ulonglong(0), ct.c_ulonglong(0)
        if self.L.bl_closure_stats(self.ctx, ct.byref(a), ct.byref(b)) != 0:
            raise RuntimeError("bl_closure_stats failed")
        return a.value, b.value

    @property
    def kernel_launches(self):
        return self.L.bl_kernel_launches(self.ctx)

    def close(self):
        if self.ctx:
            self.L.bl_finalize(self.ctx)
            self.ctx = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
