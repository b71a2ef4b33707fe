"""A batch of independent problems advanced together on the device.

``BatchSolver`` registers several Problems -- each what one control file
describes, with its own mesh, materials, time-step controls and end time --
with bl_init_batch, and advances them with bl_run_batch: one kernel per
phase over all the meshes, each mesh keeping its own dt and time on the
device.  Every mesh ends as it would running alone (bit for bit in exact
mode), mixed cells and the learned closure included.  ``sync_to_host``
updates each Problem's own arrays.
"""
import ctypes as ct

from . import abi
from ._lib import load
from .solver import SolverError


class BatchSolver:
    def __init__(self, problems, fp_mode=abi.FP_FAST):
        self.L = load()
        self.fp_mode = fp_mode
        self.launches_closed = 0     # kernel launches of contexts replaced by compaction
        self.compactions = []        # (step, meshes, elements) of each rebuild
        self._init(list(problems))

    def _init(self, problems):
        self.problems = problems
        n = len(self.problems)
        self.error = abi.Error()
        self._tabs = [p.pointer_table() for p in self.problems]
        self._sizes = (abi.Sizes * n)(*[p.sizes for p in self.problems])
        self._configs = (abi.Config * n)(*[p.config for p in self.problems])
        self._dh = (ct.c_void_p * n)(*[ct.cast(t, ct.c_void_p) for t in self._tabs])
        self.ctx = ct.c_void_p()
        ierr = self.L.bl_init_batch(ct.byref(self.ctx), n, ct.cast(self._sizes, ct.c_void_p),
                                    ct.cast(self._configs, ct.c_void_p),
                                    ct.cast(self._dh, ct.c_void_p), int(self.fp_mode),
                                    ct.byref(self.error))
        if ierr != 0:
            raise SolverError(ierr, self.error.iout, self.error.message)

    def __len__(self):
        return len(self.problems)

    def run(self, max_steps=10**9):
        """Advances every mesh until its end time (or an error, or max_steps
        steps).  Returns (ierr, per-mesh status list, steps run); each
        Problem's timestep is updated."""
        n = len(self.problems)
        ts = (abi.Timestep * n)(*[p.timestep for p in self.problems])
        status = (ct.c_int * n)()
        nsteps = ct.c_int(0)
        ierr = self.L.bl_run_batch(self.ctx, ct.cast(ts, ct.c_void_p),
                                   int(min(max_steps, 2**31 - 1)), status, ct.byref(nsteps),
                                   ct.byref(self.error))
        for p, t in zip(self.problems, ts):
            ct.memmove(ct.addressof(p.timestep), ct.addressof(t), ct.sizeof(abi.Timestep))
        return ierr, list(status), nsteps.value

    def run_compacting(self, max_steps=10**9, keep=0.5, chunk=256):
        """run() in chunks of `chunk` steps that drops finished meshes: when
        the meshes still running (before their end time, no error) hold
        fewer than `keep` of the batch's elements, their state is brought to
        the host (their own Problem arrays) and the batch is set up again
        from them alone, so that the kernels no longer launch over finished
        meshes.  Every mesh still ends as it would alone: its state passes
        through the host unchanged and the kernels are the same.  Returns
        (ierr, {id(problem): status}, steps run)."""
        everyone = list(self.problems)
        status = {id(p): 0 for p in everyone}
        done = 0
        ierr = 0
        while done < max_steps:
            ierr, st, n = self.run(max_steps=min(chunk, max_steps - done))
            for p, v in zip(self.problems, st):
                status[id(p)] = v
            done += n
            if ierr != 0 or n == 0:
                break
            alive = [p for p, v in zip(self.problems, st)
                     if v == 0 and p.timestep.time < p.config.time_end]
            if not alive:
                break
            nel_all = sum(p.nel for p in self.problems)
            nel_alive = sum(p.nel for p in alive)
            if nel_alive < keep * nel_all:
                self.sync_to_host(0)
                self.launches_closed += self.kernel_launches
                self.close()
                self.compactions.append((done, len(alive), nel_alive))
                self._init(alive)
        return ierr, status, done

    @property
    def total_launches(self):
        return self.launches_closed + self.kernel_launches

    def autotune(self):
        """Chooses the steps per graph and the node kernels' block size by
        timing each candidate from the Problems' current arrays (which it
        uploads again afterwards).  Returns (steps per graph, block size,
        {(steps, block): ms per step})."""
        n = len(self.problems)
        ts = (abi.Timestep * n)(*[p.timestep for p in self.problems])
        g, bs = ct.c_int(0), ct.c_int(0)
        ms = (ct.c_double * 9)()
        ierr = self.L.bl_autotune_batch(self.ctx, ct.cast(ts, ct.c_void_p), ct.byref(g),
                                        ct.byref(bs), ms, 9, ct.byref(self.error))
        if ierr != 0:
            raise SolverError(ierr, self.error.iout, self.error.message)
        cand = [(G, B) for G in (8, 16, 32) for B in (128, 256, 512)]
        return g.value, bs.value, dict(zip(cand, list(ms)))

    def set_closure(self, net, norm, on=True, volume_only=False):
        """The learned mixed-cell closure for every mesh of the batch (see
        Solver.set_closure)."""
        from .solver import Solver
        Solver.set_closure(self, net, norm, on, volume_only)

    def closure_stats(self):
        """(mixed-cell steps the closure saw, those it left to the plain
        closure), over all meshes."""
        from .solver import Solver
        return Solver.closure_stats(self)

    def sync_to_host(self, fid=0):
        return self.L.bl_sync_to_host(self.ctx, fid)

    def sync_to_device(self, fid=0):
        return self.L.bl_sync_to_device(self.ctx, fid)

    @property
    def stream(self):
        return self.L.bl_stream(self.ctx)

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
