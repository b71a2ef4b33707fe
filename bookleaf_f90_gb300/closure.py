"""The learned mixed-cell closure: network, sub-cell training data, training.

The reference's Lagrangian step keeps each material's volume fraction in a
mixed cell fixed (every material takes its fraction of the cell's volume
change), so two materials at different pressures in one cell never relax
towards each other.  The learned closure replaces that split for
two-material cells: a 10-64-64-2 SiLU network (``ClosureNet``; BF16
operands on the tensor cores, FP32 accumulation, trained by Adam on the
GPU) predicts each material's volume change over the step, and the device
kernel after k_lag_state applies it, or the plain closure wherever the
prediction fails its checks (see ``Solver.set_closure``).

Training data come from the same problem run at ``refine`` times the
resolution with the plain closure: the fine cells inside each coarse cell
resolve the interface, so adding up their material volumes, masses and
energies gives each coarse cell's material state (its "sub-cell" truth).
Pairs of such states a few fine steps apart give the samples: the features
of the coarse cell at the first state and the change of each material's
volume over the pair; the network learns the part of that change the plain
closure misses (``exchange``), so that a zero output is the plain closure.

Everything here runs through the library: the fine runs through
``Solver.run``, training through ``bl_mlp_train``; numpy only gathers the
snapshots into samples.
"""
import ctypes as ct

import numpy as np

from . import abi
from ._lib import load
from .setup import ic as icmod

NI, NH, NO = 10, 64, 2
NPARAM = NH * NI + NH + NH * NH + NH + NO * NH + NO
FEATURES = ("fr1", "rho1", "rho2", "p1", "p2", "cs2_1", "cs2_2", "dv", "courant", "dp_rel")


def init_params(seed=0):
    """Weights uniform in +-1/sqrt(fan_in), biases zero, in the library's
    layout W1[64][10], b1[64], W2[64][64], b2[64], W3[2][64], b3[2]."""
    rng = np.random.default_rng(seed)
    parts = []
    for rows, cols in ((NH, NI), (NH, NH), (NO, NH)):
        lim = 1.0 / np.sqrt(cols)
        parts += [rng.uniform(-lim, lim, rows * cols), np.zeros(rows)]
    return np.concatenate(parts).astype(np.float32)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _vp(a):
    return a.ctypes.data_as(ct.c_void_p)


class ClosureNet:
    """The closure network on the device (bl_mlp_*)."""

    def __init__(self, params=None, seed=0):
        self.L = load()
        self._h = ct.c_void_p()
        p = _f32(init_params(seed) if params is None else params)
        if p.size != NPARAM or self.L.bl_mlp_create(ct.byref(self._h), _vp(p)) != 0:
            raise RuntimeError("bl_mlp_create failed")

    @property
    def handle(self):
        return self._h

    def predict(self, x):
        x = _f32(x).reshape(-1, NI)
        y = np.zeros((len(x), NO), np.float32)
        if self.L.bl_mlp_predict(self._h, _vp(x), len(x), _vp(y)) != 0:
            raise RuntimeError("bl_mlp_predict failed")
        return y

    def train(self, x, t, epochs=200, batch=256, lr=1e-3, seed=0):
        """Adam over shuffled mini-batches; returns each epoch's mean loss."""
        x, t = _f32(x).reshape(-1, NI), _f32(t).reshape(-1, NO)
        losses = np.zeros(epochs, np.float32)
        if self.L.bl_mlp_train(self._h, _vp(x), _vp(t), len(x), int(epochs), int(batch),
                               float(lr), int(seed), _vp(losses)) != 0:
            raise RuntimeError("bl_mlp_train failed")
        return losses

    def params(self):
        p = np.zeros(NPARAM, np.float32)
        if self.L.bl_mlp_params(self._h, _vp(p)) != 0:
            raise RuntimeError("bl_mlp_params failed")
        return p

    def close(self):
        if self._h:
            self.L.bl_mlp_destroy(self._h)
            self._h = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- sub-cell data

def grid_index(problem, nx, ny):
    """Each element's cell of an nx x ny grid over the mesh's bounding box,
    by its centroid (call before the mesh moves)."""
    f = problem.fields
    nd = f[abi.IELND].reshape(-1, 4) - 1
    x, y = f[abi.NDX], f[abi.NDY]
    xc, yc = x[nd].mean(axis=1), y[nd].mean(axis=1)
    i = np.clip(((xc - x.min()) / (x.max() - x.min()) * nx).astype(np.int64), 0, nx - 1)
    j = np.clip(((yc - y.min()) / (y.max() - y.min()) * ny).astype(np.int64), 0, ny - 1)
    return j * nx + i


def material_sums(problem, index, ncell):
    """Volume, mass and internal energy of materials 1 and 2 in each of
    ncell cells (elements mapped by index), from pure elements and
    mixed-cell components alike; arrays of shape (ncell, 2).  Each sum runs
    over the elements (then the components) in their order (np.bincount
    accumulates in input order, as np.add.at does, many times faster)."""
    f = problem.fields
    ielmat = f[abi.IELMAT]
    pure = ielmat > 0
    cell, mat = index[pure], ielmat[pure] - 1
    keep = mat < 2
    bins = [2 * cell[keep] + mat[keep]]
    el_m = f[abi.ELMASS][pure][keep]
    vols = [f[abi.ELVOLUME][pure][keep]]
    mass = [el_m]
    ener = [el_m * f[abi.ELENERGY][pure][keep]]
    if problem.sizes.ncp > 0:
        cp_el = np.repeat(f[abi.IMXEL][:problem.sizes.nmx] - 1, f[abi.IMXNCP][:problem.sizes.nmx])
        cmat = f[abi.ICPMAT][:len(cp_el)] - 1
        keep = cmat < 2
        bins.append(2 * index[cp_el[keep]] + cmat[keep])
        cm = f[abi.CPMASS][:len(cp_el)][keep]
        vols.append(f[abi.CPVOLUME][:len(cp_el)][keep])
        mass.append(cm)
        ener.append(cm * f[abi.CPENERGY][:len(cp_el)][keep])
    b = np.concatenate(bins)
    out = [np.bincount(b, weights=np.concatenate(w), minlength=2 * ncell).reshape(ncell, 2)
           for w in (vols, mass, ener)]
    return out[0], out[1], out[2]


def features(config, V, M, E, dvol, dt):
    """The closure's ten features (FEATURES) of cells with material sums
    V, M, E (ncell, 2), relative volume change dvol and step dt, as the
    device kernel forms them from a mixed cell's components."""
    Vc = V.sum(axis=1)
    rho = M / V
    e = E / M
    p = np.empty_like(rho)
    c2 = np.empty_like(rho)
    for k in range(2):
        p[:, k], c2[:, k] = icmod.eos(config, np.full(len(V), k + 1), rho[:, k], e[:, k])
    return np.stack([V[:, 0] / Vc, rho[:, 0], rho[:, 1], p[:, 0], p[:, 1], c2[:, 0], c2[:, 1],
                     dvol, dt * np.sqrt(np.maximum(c2[:, 0], c2[:, 1]) / Vc),
                     (p[:, 0] - p[:, 1]) / (np.abs(p[:, 0]) + np.abs(p[:, 1]) + 1e-300)], axis=1)


def subcell_samples(make, nx, ny, refine=4, lags=(1, 2, 4), fp_mode=abi.FP_FAST,
                    min_fraction=1e-4, min_change=1e-8):
    """Samples of the learned closure from a plain run at ``refine`` times
    the resolution nx x ny of the problem ``make(nx, ny) -> (deck,
    material_fraction)`` (e.g. configs.sod_interface).  The run is gathered
    onto the coarse cells after every fine step, and each pair of states
    ``lag`` fine steps apart (for every lag in lags: the coarse step spans
    about ``refine`` fine steps once dt follows the CFL limit, one while it
    still grows from dt_initial) gives, for each coarse two-material cell,
    a sample.  Returns (X, D, truth): X the features at the first state of
    the pair, D (n, 2) the materials' volume changes over the pair as
    fractions of the cell's volume, and truth the coarse cells' material
    volumes and masses (V, M) at the end of the run.  Cells count as mixed
    while both materials fill more than min_fraction of them; pairs in which
    no material's volume changes by min_change of the cell are skipped."""
    from .setup import Problem
    from .solver import Solver
    deck, fraction = make(nx * refine, ny * refine)
    pf = Problem.from_deck(deck, material_fraction=fraction)
    index = grid_index(pf, nx, ny)
    ncell = nx * ny
    s = Solver(pf, fp_mode=fp_mode)
    X, D = [], []
    try:
        s.sync_to_host(0)
        hist = [material_sums(pf, index, ncell) + (pf.timestep.time,)]
        # masses never change: after the first download only the volumes
        # and energies are read back
        moving = (abi.ELVOLUME, abi.ELENERGY) + ((abi.CPVOLUME, abi.CPENERGY)
                                                 if pf.sizes.ncp > 0 else ())
        while pf.timestep.time < pf.config.time_end:
            ierr, _ = s.run(max_steps=1, history=False)
            if ierr != 0:
                raise RuntimeError("fine run failed: " + s.error.message)
            for fid in moving:
                s.sync_to_host(fid)
            cur = material_sums(pf, index, ncell) + (pf.timestep.time,)
            hist = (hist + [cur])[-(max(lags) + 1):]
            for lag in lags:
                if lag >= len(hist):
                    continue
                V0, M0, E0, t0 = hist[-1 - lag]
                Vc0 = V0.sum(axis=1)
                fr = V0[:, 0] / np.maximum(Vc0, 1e-300)
                d = (cur[0] - V0) / np.maximum(Vc0, 1e-300)[:, None]
                sel = (fr > min_fraction) & (fr < 1.0 - min_fraction)
                sel &= np.abs(d).max(axis=1) > min_change
                if np.any(sel):
                    X.append(features(pf.config, V0[sel], M0[sel], E0[sel],
                                      d[sel].sum(axis=1), cur[3] - t0))
                    D.append(d[sel])
    finally:
        s.close()
    return np.concatenate(X), np.concatenate(D), hist[-1][:2]


# ---------------------------------------------------------------- training

def exchange(X, D):
    """The volume each material gains beyond its volume-fraction share of
    the cell's change (the network's target; sums to zero over a cell)."""
    fr = np.stack([X[:, 0], 1.0 - X[:, 0]], axis=1)
    return D - fr * X[:, 7:8]


def fit_norm(X, D):
    """The device kernel's 22-float standardisation: feature means, inverse
    standard deviations, the output scale (the root mean square of the
    exchanged volumes) and, last, the volume-conservation tolerance on the
    outputs (set by ``calibrate``)."""
    mu = X.mean(axis=0)
    sd = X.std(axis=0)
    inv = np.where(sd > 1e-12 * np.maximum(np.abs(mu), 1e-300), 1.0 / np.maximum(sd, 1e-300), 1.0)
    sig = float(np.sqrt(np.mean(exchange(X, D) ** 2))) or 1.0
    return np.concatenate([mu, inv, [sig, 0.0]]).astype(np.float32)


def standardise(X, D, norm):
    """Network inputs and targets for features X and volume changes D."""
    x = ((X.astype(np.float32) - norm[:NI]) * norm[NI:2 * NI]).astype(np.float32)
    t = None if D is None else (exchange(X, D) / norm[2 * NI]).astype(np.float32)
    return x, t


def calibrate(net, X, norm, factor=4.0):
    """Sets the conservation tolerance norm[21] to ``factor`` times the root
    mean square of the outputs' sum over the samples X (it is zero for a
    perfect fit): a prediction that misses conservation by more than the
    network does on its own training data is rejected."""
    x, _ = standardise(X, None, norm)
    y = net.predict(x)
    norm = norm.copy()
    norm[2 * NI + 1] = max(factor * float(np.sqrt(np.mean((y[:, 0] + y[:, 1]) ** 2))), 1e-3)
    return norm


def train(X, D, epochs=300, batch=256, lr=2e-3, seed=0):
    """A network trained on samples (X, D): returns (net, norm, losses)."""
    norm = fit_norm(X, D)
    x, t = standardise(X, D, norm)
    net = ClosureNet(seed=seed)
    losses = net.train(x, t, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return net, calibrate(net, X, norm), losses


# ---------------------------------------------------------------- evaluation

def mixed_errors(problem, index, truth, cells):
    """Errors of a coarse run's material state against the sub-cell truth
    (V, M) in the given cells: (mean |fr1 - fr1_true|, mean relative
    density error of material 1, of material 2)."""
    V, M, _ = material_sums(problem, index, len(truth[0]))
    Vt, Mt = truth
    fr = V[cells, 0] / V[cells].sum(axis=1)
    frt = Vt[cells, 0] / Vt[cells].sum(axis=1)
    rho = M[cells] / V[cells]
    rhot = Mt[cells] / Vt[cells]
    rel = np.abs(rho - rhot) / rhot
    return float(np.mean(np.abs(fr - frt))), float(np.mean(rel[:, 0])), float(np.mean(rel[:, 1]))


def interface_positions(problem, index, nx, ny):
    """Per row of the coarse grid, the position of the interface as the
    share of the row's volume that is material 1 times the tube's length
    (material 1 fills the left; exact for an interface across the rows)."""
    V, _, _ = material_sums(problem, index, nx * ny)
    x = problem.fields[abi.NDX]
    row = V.reshape(ny, nx, 2).sum(axis=1)
    return x.min() + row[:, 0] / row.sum(axis=1) * (x.max() - x.min())


def against_plain(learned, plain, index, nx, ny):
    """The learned closure's run against the plain closure's on the same
    mesh: (largest shift of the interface in any row, in cells; relative L1
    difference of the mixed cells' densities; of all cells' densities)."""
    dx = (plain.fields[abi.NDX].max() - plain.fields[abi.NDX].min()) / nx
    shift = np.max(np.abs(interface_positions(learned, index, nx, ny) -
                          interface_positions(plain, index, nx, ny))) / dx
    el = plain.fields[abi.IMXEL][:plain.sizes.nmx] - 1
    rl, rp = learned.fields[abi.ELDENSITY], plain.fields[abi.ELDENSITY]
    return (float(shift), float(np.sum(np.abs(rl[el] - rp[el])) / np.sum(np.abs(rp[el]))),
            float(np.sum(np.abs(rl - rp)) / np.sum(np.abs(rp))))


def cell_density_error(problem, index, truth, cells):
    """Relative L1 error of the given cells' densities (the cell's mass over
    its volume) against the sub-cell truth (V, M)."""
    el = problem.fields[abi.IMXEL][:problem.sizes.nmx] - 1
    Vt, Mt = truth
    rt = Mt[cells].sum(axis=1) / Vt[cells].sum(axis=1)
    r = problem.fields[abi.ELDENSITY][el]
    return float(np.sum(np.abs(r - rt)) / np.sum(rt))


def main(argv=None):
    """A small end-to-end run: sub-cell samples of one tilted two-material
    tube, a short training, then that tube coarse with the learned closure
    for a number of steps; prints what it did.  Used as the profiling case
    of the closure's kernels (k_mlp_grad, k_mix_closure)."""
    import argparse
    import functools
    from .setup import Problem, configs
    from .solver import Solver
    ap = argparse.ArgumentParser(prog="python -m bookleaf_f90_gb300.closure")
    ap.add_argument("--nx", type=int, default=160)
    ap.add_argument("--epochs", type=int, default=2)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--tilt", type=float, default=0.2)
    ap.add_argument("--state", type=float, default=0.5)
    a = ap.parse_args(argv)
    ny = max(1, a.nx // 10)
    make = functools.partial(configs.sod_interface, time_end=0.02, amplitude=0.0, periods=0,
                             tilt=a.tilt, rho_right=a.state, p_right=a.state)
    X, D, _ = subcell_samples(make, a.nx, ny)
    net, norm, losses = train(X, D, epochs=a.epochs)
    deck, fraction = make(a.nx, ny)
    p = Problem.from_deck(deck, material_fraction=fraction)
    s = Solver(p)
    s.set_closure(net, norm)
    ierr, _ = s.run(max_steps=a.steps, history=False)
    seen, rejected = s.closure_stats()
    print("samples %d, loss %.4g -> %.4g, %d steps (ierr %d), closure cells %d, rejected %d"
          % (len(X), losses[0], losses[-1], p.timestep.nstep, ierr, seen, rejected))
    s.close()
    net.close()
    return ierr


if __name__ == "__main__":
    raise SystemExit(main())
