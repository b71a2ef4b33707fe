"""Benchmark of the BookLeaf hydro hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload sedov|noh|noh-polar|noh-eul|sod|ensemble|closure|closure-ensemble]
                    [--size S]

A step is one pass of the hot path (getdt + lagstep, + alestep for Eulerian
workloads) over the whole mesh.  The default workload is the Sedov blast on
a 512x512 quarter domain, Lagrangian, FP64 (the configuration the metric is
quoted on).  Inputs are synthetic: the deck is generated in the reference's
namelist format (bookleaf_f90_gb300/setup/configs.py).

value      zone-cycles/s with the state resident in HBM: K steps of the
           device-resident time loop (bl_run, CUDA graphs), timed with CUDA
           events on the library's stream.
e2e        the same metric through the reference-facing C-ABI with host
           buffers: bl_init (upload of every registered host field), K calls
           each of bl_getdt/bl_lagstep(/bl_alestep) and bl_sync_to_host of
           the whole state, all inside the timed region.
roofline   the dominant kernel (edge viscosity + dt, k_getdt) against the
           measured HBM copy bandwidth, with algorithmic bytes per zone
           (each field read once plus each field written once); "fp64"
           reports the binding FP64 issue roof.
cpu_baseline  the CPU restatement on this host's cores, a bounded sample
           of the same workload.

Under torchrun (N>1) every rank advances its own replica (the plain path does
not shard without halo exchange); value is the sum over ranks divided by
the slowest rank's time.
"""
import argparse
import json

import numpy as np
import os
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

# algorithmic bytes per zone-cycle: each field a phase reads counted once
# plus each field it writes counted once (FP64 8 B, INT32 4 B, node fields
# per node)
B_LAG = 724
B_EUL = 1628
B_GETDT = 164
# the headline metric, printed by both arms
METRIC = "zone-cycles/s FP64 (1 GB300, %HBM roof); batched+MLP vs plain GPU at stated L1 err"


def load_profile(name="k_getdt_current.json"):
    """The committed summary of the latest single-kernel ncu capture of
    k_getdt (profiles/k_getdt_current.json): its FP64-pipe thread
    instructions per zone and DRAM bytes per launch, with the command and
    mesh size they were taken at; None where absent."""
    path = os.path.join(HERE, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def workload_deck(name, size):
    from bookleaf_f90_gb300 import configs
    if name == "ensemble":
        return None, "ensemble_%d_eulerian_sod_sedov" % (size or 512), True
    if name == "closure-ensemble":
        return None, "closure_ensemble_%d_sod2mat_tilted" % (size or 64), False
    if name == "closure":
        n = size or 800
        return None, "sod2mat_tilted_%dx%d_learned_closure" % (n, max(1, n // 10)), False
    if name == "sedov":
        # the reference's Sedov decks set the hourglass filter kappaall=0.01
        # (input/sedov_lag_small); at 512x512 the sub-zonal pressure force
        # (pmeritall=0.1) is needed as well for the mesh to reach t = 1
        n = size or 512
        return (configs.sedov(n, kappa=0.01, pmerit=0.1),
                "sedov_%dx%d_lagrangian_t1_hg0.01_sp0.1" % (n, n), False)
    if name == "noh":
        return configs.noh(size or 2048), "noh_%dx%d_lagrangian" % (size or 2048, size or 2048), False
    if name == "noh-polar":
        # the reference's own Noh mesh family (input/noh_small, noh_large:
        # the polar quarter annulus); --size sets the radial cells, 0.4x
        # around.  300 x 120 is the largest tried that reaches t = 0.6:
        # from 900 x 360 (and noh_large's 1800 x 720) the reference's method
        # stops with dt < dt_min (the oracle at 900 x 360 at step 2,839,
        # as the device)
        nr = size or 300
        return (configs.noh_polar(nr, max(1, (nr * 2) // 5)),
                "noh_polar_%dx%d_lagrangian_t0.6" % (nr, max(1, (nr * 2) // 5)), False)
    if name == "noh-eul":
        return configs.noh(size or 2048, eulerian=True), "noh_%dx%d_eulerian" % (size or 2048, size or 2048), True
    if name == "sod":
        return configs.sod(size or 400, max(1, (size or 400) // 10)), "sod_%dx%d_lagrangian" % (
            size or 400, max(1, (size or 400) // 10)), False
    raise SystemExit("unknown workload " + name)


def load_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


_NVML_REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
                 0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}


class _Nvml:
    """Read-only NVML queries through ctypes (the driver's libnvidia-ml):
    SM clock, its maximum and the active clock-event reasons of one GPU."""

    def __init__(self, torch_index):
        import ctypes as ct
        self.ct = ct
        self.lib = ct.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.dev = ct.c_void_p()
        rc = -1
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(torch_index).uuid)
            uuid = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
            rc = self.lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ct.byref(self.dev))
        except Exception:
            rc = -1
        if rc != 0:
            rc = self.lib.nvmlDeviceGetHandleByIndex_v2(ct.c_uint(torch_index), ct.byref(self.dev))
        if rc != 0:
            raise OSError("no NVML handle")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        ct = self.ct
        clk, mx, rs = ct.c_uint(0), ct.c_uint(0), ct.c_ulonglong(0)
        self.lib.nvmlDeviceGetClockInfo(self.dev, 1, ct.byref(clk))       # NVML_CLOCK_SM
        self.lib.nvmlDeviceGetMaxClockInfo(self.dev, 1, ct.byref(mx))
        self.reasons_fn(self.dev, ct.byref(rs))
        return clk.value, mx.value, rs.value


class ClockSampler:
    """SM clock and clock-event reasons DURING the timed region: a thread
    polls NVML every 0.5 ms between __enter__ and __exit__ (the library's
    calls release the interpreter lock), so that even a region of a few
    milliseconds gets samples; one sample is also taken at each end.  Falls
    back to one nvidia-smi query at each end where NVML cannot be loaded."""

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.samples = []
        self.how = "nvml poll 0.5 ms"
        try:
            self.nv = _Nvml(gpu_index)
        except (OSError, AttributeError):
            self.nv = None
            self.how = "nvidia-smi at both ends"

    def _smi(self):
        try:
            out = subprocess.run(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=clocks.sm,clocks.max.sm,"
                 "clocks_event_reasons.active", "--format=csv,noheader,nounits"],
                capture_output=True, text=True, timeout=10).stdout.strip().split(",")
            self.samples.append((float(out[0]), float(out[1]), int(out[2].strip(), 16)))
        except Exception:
            pass

    def _poll(self):
        while not self.stop.is_set():
            self.samples.append(self.nv.sample())
            time.sleep(0.0005)

    def __enter__(self):
        self.stop = threading.Event()
        if self.nv is None:
            self._smi()
            return self
        self.samples.append(self.nv.sample())
        self.t = threading.Thread(target=self._poll, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        if self.nv is None:
            self._smi()
            return
        self.stop.set()
        self.t.join()
        self.samples.append(self.nv.sample())

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(s[0] for s in self.samples)
        reasons = set()
        for s in self.samples:
            for bit, name in _NVML_REASONS.items():
                if s[2] & bit:
                    reasons.add(name)
        return {"sm_mhz": sm[len(sm) // 2], "sm_min_mhz": sm[0],
                "sm_max_mhz": max(s[1] for s in self.samples),
                "reasons": sorted(reasons), "samples": len(self.samples), "how": self.how}


def cpu_sample(deck, steps, warmup=1):
    """The CPU restatement advancing `steps` steps of the workload from
    t = 0, after `warmup` untimed steps on a copy of the same initial state;
    returns (zone-cycles/s, seconds).  Runs in a spawned worker process."""
    sys.path.insert(0, HERE)
    from bookleaf_f90_gb300 import Problem
    from oracle.oracle import Oracle
    p = Problem.from_deck(deck)
    if warmup > 0:
        q = p.copy()
        oq = Oracle(q)
        for _ in range(warmup):
            if oq.step(q.timestep) != 0:
                break
        del oq, q
    o = Oracle(p)
    t0 = time.perf_counter()
    n = 0
    for _ in range(steps):
        if o.step(p.timestep) != 0:
            break
        n += 1
    t = time.perf_counter() - t0
    return p.nel * n / t, t


def cpu_baseline(deck, nel, target_s=12.0, cores=1, steps=0, warmup=1):
    """The workload on the host's cores (spawned workers, one independent
    replica each): `steps` steps from t = 0, or with steps = 0 as many as
    fill about target_s seconds (calibrated on one step).  Returns (summed
    zone-cycles/s, steps, slowest worker's seconds)."""
    import multiprocessing as mp
    from oracle import oracle as orc
    orc.build()
    ctx = mp.get_context("spawn")
    if steps <= 0:
        with ctx.Pool(1) as pool:
            rate, t = pool.apply(cpu_sample, (deck, 1, 0))
        steps = max(2, int(target_s * rate / nel))
    with ctx.Pool(cores) as pool:
        res = pool.starmap(cpu_sample, [(deck, steps, warmup)] * cores)
    rate = sum(r for r, _ in res)
    return rate, steps, max(t for _, t in res)


def run_ensemble(args, torch, rank=0, world=1):
    """The batched ensemble (--workload ensemble; --size = number of meshes,
    default 512): every mesh of configs.ensemble advanced together by
    bl_run_batch, in the floating-point mode --fp selects (mixed: the
    demoted form), against the same meshes run one after another through
    the plain per-mesh device loop (bl_run) in FP64 (fast; exact if --fp
    exact).  Both run every mesh from t = 0 to its own end time (--steps K
    > 0: K steps instead), timed with CUDA events, after W warm-up steps and
    a re-upload of the initial state; the batch runs in chunks of 256 steps
    and is set up again from the meshes still running whenever they hold
    less than half its elements (BatchSolver.run_compacting).  The batch's
    L1 errors against the FP64 per-mesh results are reported per mesh at
    the end time and after 50 steps of both (the same step count).  Under
    torchrun each rank takes its share of the meshes (replicas.shard: by
    elements times resolution, the step count growing with it) and runs
    them as one GPU does; the rates are the zone-cycles of all ranks over
    the slowest rank's time, and rank 0 gathers the per-mesh errors (the
    ensemble is fixed: strong scaling).  Returns the line on rank 0, None
    on the others."""
    from bookleaf_f90_gb300 import BatchSolver, Problem, Solver, abi, configs
    import ctypes as ct
    n = args.size or 512
    seed = 20240607
    K = args.steps if args.steps > 0 else 10**9
    W = max(1, args.warmup)
    fp = {"exact": abi.FP_EXACT, "fast": abi.FP_FAST, "mixed": abi.FP_MIXED}[args.fp]
    fp_plain = abi.FP_EXACT if args.fp == "exact" else abi.FP_FAST
    from bookleaf_f90_gb300.replicas import gather_to_root, job_rate, shard
    items = configs.ensemble(n, seed=seed)
    weights = [m["nx"] * m["ny"] * max(m["nx"], m["ny"]) for _, m in items]
    mine = shard(weights, world, rank)
    items = [items[i] for i in mine]
    dev = "cuda" if world > 1 else None

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    t0 = time.perf_counter()
    probs = [Problem.from_deck(d) for d, _ in items]
    setup_s = time.perf_counter() - t0
    nels = [p.nel for p in probs]
    init = [({fid: a.copy() for fid, a in p.fields.items()}, p.timestep.copy()) for p in probs]

    def restore(p, i):
        for fid, a in init[i][0].items():
            np.copyto(p.fields[fid], a)
        ct.memmove(ct.addressof(p.timestep), ct.addressof(init[i][1]), ct.sizeof(abi.Timestep))

    def l1s(pa, pb):
        out = []
        for f in (abi.ELDENSITY, abi.ELENERGY):
            a, b = pa.fields[f], pb.fields[f]
            out.append(float(np.sum(np.abs(a - b)) / max(np.sum(np.abs(b)), 1e-300)))
        du = (np.abs(pa.fields[abi.NDU] - pb.fields[abi.NDU])
              + np.abs(pa.fields[abi.NDV] - pb.fields[abi.NDV]))
        un = np.abs(pb.fields[abi.NDU]) + np.abs(pb.fields[abi.NDV])
        out.append(float(np.sum(du) / max(np.sum(un), 1e-300)))
        return out

    def l1_summary(rows):
        a = np.array(rows)
        names = ("density", "energy", "velocity")
        return {nm: {"max": float(a[:, k].max()), "median": float(np.median(a[:, k]))}
                for k, nm in enumerate(names)}

    # ---- L1 after 50 steps: the batch in its mode against the batch in
    # FP64 (equal, mesh by mesh, to each mesh alone: tests/test_gpu_batch.py)
    rows_50 = None
    if fp != fp_plain:
        ref = [p.copy() for p in probs]
        bm = BatchSolver(probs, fp_mode=fp)
        assert bm.run(max_steps=50)[0] == 0, bm.error.message
        bm.sync_to_host(0)
        bm.close()
        bf = BatchSolver(ref, fp_mode=fp_plain)
        assert bf.run(max_steps=50)[0] == 0, bf.error.message
        bf.sync_to_host(0)
        bf.close()
        rows_50 = [l1s(a, b) for a, b in zip(probs, ref)]
        del ref
        for i, p in enumerate(probs):
            restore(p, i)

    # ---- batched: autotune (steps per graph, node block size), warm up
    b = BatchSolver(probs, fp_mode=fp)
    tg, tb, tms = b.autotune()
    ierr, _, _ = b.run(max_steps=W)
    assert ierr == 0, b.error.message
    for i, p in enumerate(probs):
        restore(p, i)
    b.sync_to_device(0)
    stream = torch.cuda.ExternalStream(b.stream)
    n0 = [p.timestep.nstep for p in probs]
    l0 = b.total_launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record(stream)
        ierr, status, nsteps = b.run_compacting(max_steps=K)
        e1.record(torch.cuda.ExternalStream(b.stream))
        e1.synchronize()
    assert ierr == 0, b.error.message
    ms_b = e0.elapsed_time(e1)
    steps_b = [p.timestep.nstep - s0 for p, s0 in zip(probs, n0)]
    zc_b = sum(nel * k for nel, k in zip(nels, steps_b))
    done = sum(1 for p in probs if p.timestep.time >= p.config.time_end)
    launches = b.total_launches - l0
    compactions = list(b.compactions)
    b.sync_to_host(0)
    b.close()
    batch_final = [p.copy() for p in probs]
    value, t_b, _ = job_rate(ms_b, zc_b, device=dev)
    # ---- e2e: batch set-up from the host arrays, the same run, full download
    for i, p in enumerate(probs):
        restore(p, i)
    barrier()
    t0 = time.perf_counter()
    be = BatchSolver(probs, fp_mode=fp)
    ierr, _, ne = be.run_compacting(max_steps=K)
    be.sync_to_host(0)
    t1 = time.perf_counter()
    assert ierr == 0, be.error.message
    zc_e = sum(nel * p.timestep.nstep for nel, p in zip(nels, probs))
    h2d = sum(a.nbytes for p in probs for a in p.fields.values())
    be.close()
    e2e_value, _, _ = job_rate((t1 - t0) * 1e3, zc_e, device=dev)
    # ---- plain: each mesh alone in FP64
    barrier()
    ms_p, zc_p = 0.0, 0
    rows_end, dt_end = [], []
    for i, p in enumerate(probs):
        restore(p, i)
        s = Solver(p, fp_mode=fp_plain)
        ierr, _ = s.run(max_steps=W, ts=p.timestep.copy(), history=False)
        assert ierr == 0, s.error.message
        restore(p, i)
        s.sync_to_device(0)
        st = torch.cuda.ExternalStream(s.stream)
        q0 = torch.cuda.Event(enable_timing=True)
        q1 = torch.cuda.Event(enable_timing=True)
        ts = p.timestep.copy()
        q0.record(st)
        ierr, _ = s.run(max_steps=K, ts=ts, history=False)
        q1.record(st)
        q1.synchronize()
        assert ierr == 0, s.error.message
        ms_p += q0.elapsed_time(q1)
        zc_p += p.nel * (ts.nstep - init[i][1].nstep)
        s.sync_to_host(0)
        p.timestep = ts
        rows_end.append(l1s(batch_final[i], p))
        dt_end.append(abs(batch_final[i].timestep.time - ts.time) / max(ts.dt, 1e-300))
        s.close()
    plain, _, _ = job_rate(ms_p, zc_p, device=dev)
    clocks = clk.summary()
    parts = gather_to_root({"rows_end": rows_end, "dt_end": dt_end, "rows_50": rows_50,
                            "steps": steps_b, "done": done, "launches": launches,
                            "compactions": compactions, "nels": nels, "nsteps": nsteps,
                            "h2d": h2d, "ne": ne, "setup_s": setup_s, "ms_p": ms_p,
                            "clocks": clocks})
    if rank != 0:
        return None
    rows_end = [r for q in parts for r in q["rows_end"]]
    dt_end = [d for q in parts for d in q["dt_end"]]
    l1_50 = (l1_summary([r for q in parts for r in q["rows_50"]])
             if parts[0]["rows_50"] is not None else None)
    steps_b = [k for q in parts for k in q["steps"]]
    nels = [k for q in parts for k in q["nels"]]
    done = sum(q["done"] for q in parts)
    launches = sum(q["launches"] for q in parts)
    nsteps = max(q["nsteps"] for q in parts)
    ne = max(q["ne"] for q in parts)
    h2d = sum(q["h2d"] for q in parts)
    setup_s = max(q["setup_s"] for q in parts)
    ms_p = max(q["ms_p"] for q in parts)
    hbm_peak, peak_kind = load_peaks()
    achieved = value * B_EUL / 1e9
    return {"metric": METRIC, "what": "batched ensemble vs the plain per-mesh FP64 GPU path",
            "value": value, "unit": "zone-cycles/s", "n_gpus": world, "steps": nsteps,
            "warmup": W, "ms_per_step": t_b / max(1, nsteps), "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None,
            "dtype": "f64" if fp != abi.FP_MIXED else "f64+f32 (mixed)", "data": "synthetic",
            "config": {"workload": "ensemble_%d_eulerian_sod_sedov" % n, "instances": n,
                       "seed": seed, "nel_total": sum(nels), "nel_min": min(nels),
                       "nel_max": max(nels), "fp_mode": args.fp,
                       "meshes_at_end_time": done,
                       "timed": ("every mesh from t=0 to its own end time (%d to %d steps)"
                                 % (min(steps_b), max(steps_b))) if K >= 10**9 else
                                "%d steps from t=0" % nsteps,
                       "loop": "bl_run_batch, CUDA graphs of %d steps, in chunks of 256 "
                               "steps; the batch is set up again from the meshes still "
                               "running when they hold less than half its elements "
                               "(BatchSolver.run_compacting)" % tg,
                       "compactions": [{"after_step": a, "meshes": m, "elements": e}
                                       for a, m, e in parts[0]["compactions"]],
                       "autotune": {"graph_steps": tg, "node_block": tb,
                                    "ms_per_step": {"%d,%d" % k: v for k, v in tms.items()}},
                       "setup_s": setup_s,
                       "shards": {"ranks": world,
                                  "meshes": [len(q["nels"]) for q in parts],
                                  "elements": [sum(q["nels"]) for q in parts],
                                  "how": "replicas.shard: longest first by nx*ny*max(nx,ny), "
                                         "no exchange; rank 0's compactions and autotune "
                                         "shown"}},
            "plain_per_mesh": {"value": plain, "unit": "zone-cycles/s", "ms_total": ms_p,
                               "fp_mode": "exact" if fp_plain == abi.FP_EXACT else "fast",
                               "how": "each mesh alone through bl_run in FP64, the same run "
                                      "from t=0, CUDA events, times summed"},
            "batched_over_plain": value / plain,
            "l1_vs_plain_fp64": {"at_end_time": l1_summary(rows_end),
                                 "end_time_offset_in_dt_max": float(max(dt_end)),
                                 "after_50_steps": l1_50,
                                 "how": "per mesh: sum|batch - plain| / sum|plain| of density, "
                                        "specific energy and the velocity field; max and "
                                        "median over the meshes"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                         "peak_kind": peak_kind,
                         "note": "algorithmic bytes 1628 B per zone-cycle (Eulerian); the "
                                 "FP64 issue rate, not HBM, bounds the path"},
            "e2e": {"value": e2e_value, "unit": "zone-cycles/s",
                    "h2d_bytes_per_step": int(h2d / max(1, ne)),
                    "d2h_bytes_per_step": int(h2d / max(1, ne)),
                    "note": "bl_init_batch from the host arrays + %d steps + full download, "
                            "wall clock" % ne},
            "gpu_launches": launches, "clocks": parts[0]["clocks"]}


# Two-material Sod tubes for the learned closure (pressure and density of
# the right state s, planar interface tilted by t): the cases the network is
# trained on (sub-cell data of 4x-refined runs at 160x16) and the one it is
# measured on.  The literal sinusoidal two-material Sod (amplitude 0.02, 8
# periods, right state rho 0.125, p 0.1) stops with dt < dt_min under the
# plain closure, which gives mixed cells neither artificial viscosity nor
# hourglass control; the line records where.
CLOSURE_TRAIN = [(t, s) for t in (0.1, 0.3, 0.4) for s in (0.5, 0.6)] + [(0.1, 0.4), (0.3, 0.4)]
CLOSURE_TEST = (0.2, 0.5)
# the coarse meshes of the training runs, with their cases (at 320x32 the
# refined run of tilt 0.3, state 0.4 stops with dt < dt_min)
CLOSURE_TRAIN_MESHES = [((160, 16), CLOSURE_TRAIN),
                        ((320, 32), [c for c in CLOSURE_TRAIN if c != (0.3, 0.4)])]


def _closure_case(case, nx, ny, time_end=0.2):
    from bookleaf_f90_gb300 import configs
    tilt, st = case
    return configs.sod_interface(nx, ny, time_end=time_end, amplitude=0.0, periods=0, tilt=tilt,
                                 rho_right=st, p_right=st)


def run_closure(args, torch):
    """The learned mixed-cell closure (--workload closure; --size = cells
    across the tube, default 800, with size / 10 rows; the 4x-refined plain
    run stops with dt < dt_min from 4800 cells across): the network is
    trained on the GPU on sub-cell data of 4x-refined plain runs (160x16 and
    320x32 meshes, CLOSURE_TRAIN_MESHES), then the held-out interface is run to t = 0.2
    with the plain and with the learned closure, and 4x refined with the
    plain closure (the sub-cell truth, and the cost the coarse learned run
    replaces).  Each run is timed whole with CUDA events on its stream after
    W warm-up steps and a re-upload of the initial state."""
    import functools
    from bookleaf_f90_gb300 import Problem, Solver, abi, closure, configs
    fp = {"exact": abi.FP_EXACT, "fast": abi.FP_FAST, "mixed": abi.FP_MIXED}[args.fp]
    nx = args.size or 800
    ny = max(1, nx // 10)
    W = max(1, args.warmup)
    t0 = time.perf_counter()
    Xs, Ds = [], []
    for (tx, ty), train_cases in CLOSURE_TRAIN_MESHES:
        for case in train_cases:
            X, D, _ = closure.subcell_samples(functools.partial(_closure_case, case), tx, ty,
                                              fp_mode=fp)
            Xs.append(X)
            Ds.append(D)
    X, D = np.concatenate(Xs), np.concatenate(Ds)
    t1 = time.perf_counter()
    net, norm, losses = closure.train(X, D, epochs=100)
    t2 = time.perf_counter()

    def timed(p, learned, limit, volume_only=False, may_fail=False):
        s = Solver(p, fp_mode=fp)
        if learned:
            s.set_closure(net, norm, volume_only=volume_only)
        init = {fid: arr.copy() for fid, arr in p.fields.items()}
        ts0 = p.timestep.copy()
        ierr, _ = s.run(max_steps=W, ts=p.timestep.copy(), history=False)
        assert ierr == 0, s.error.message
        for fid, arr in init.items():
            np.copyto(p.fields[fid], arr)
        s.sync_to_device(0)
        c0 = s.closure_stats()
        l0 = s.kernel_launches
        ts = ts0.copy()
        stream = torch.cuda.ExternalStream(s.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with ClockSampler(torch.cuda.current_device()) as clk:
            e0.record(stream)
            ierr, _ = s.run(max_steps=limit, history=False, ts=ts)
            e1.record(stream)
            e1.synchronize()
        if ierr != 0 and may_fail:
            out = {"failed": s.error.message.strip(), "time": ts.time,
                   "steps": ts.nstep - ts0.nstep}
            s.close()
            return out
        assert ierr == 0, s.error.message
        assert ts.time >= p.config.time_end, "no end in %d steps" % limit
        p.timestep = ts
        s.sync_to_host(0)
        c1 = s.closure_stats()
        out = {"ms": e0.elapsed_time(e1), "steps": ts.nstep - ts0.nstep, "time": ts.time,
               "launches": s.kernel_launches - l0,
               "closure_cells": c1[0] - c0[0], "closure_rejected": c1[1] - c0[1],
               "clocks": clk.summary()}
        out["rate"] = p.nel * out["steps"] / (out["ms"] * 1e-3)
        s.close()
        return out

    deck, frac = _closure_case(CLOSURE_TEST, nx, ny)
    pp = Problem.from_deck(deck, material_fraction=frac)
    pl = pp.copy()
    pv = pp.copy()
    pe = pp.copy()
    idx = closure.grid_index(pp, nx, ny)
    cells = idx[pp.fields[abi.IMXEL][:pp.sizes.nmx] - 1]
    rp = timed(pp, False, 20000)
    rl = timed(pl, True, 20000)
    rv = timed(pv, True, 20000, volume_only=True)
    # e2e: the host arrays registered (bl_init uploads them), the closure
    # set, the run through the device loop, the whole state downloaded
    h2d = sum(a.nbytes for a in pe.fields.values())
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    se = Solver(pe, fp_mode=fp)
    se.set_closure(net, norm)
    ierr_e, _ = se.run(max_steps=20000, history=False)
    se.sync_to_host(0)
    t5 = time.perf_counter()
    assert ierr_e == 0, se.error.message
    ne = pe.timestep.nstep
    se.close()
    # the same interface refined (4x by default), plain: the sub-cell
    # truth at the end.  The plain closure itself stops with dt < dt_min on
    # this interface from about 3,200 cells across (its mixed cells get no
    # artificial viscosity); the line then records where, and the errors
    # against the truth are absent (the comparison with the plain closure
    # at the workload's own size stands).
    t3 = time.perf_counter()
    R = args.refine or 4
    deck4, frac4 = _closure_case(CLOSURE_TEST, R * nx, R * ny)
    pf = Problem.from_deck(deck4, material_fraction=frac4)
    fsetup = time.perf_counter() - t3
    fidx = closure.grid_index(pf, nx, ny)
    rf = timed(pf, False, 40000, may_fail=True)
    shift_v, l1m_v, l1a_v = closure.against_plain(pv, pp, idx, nx, ny)
    shift, l1_mixed, l1_all = closure.against_plain(pl, pp, idx, nx, ny)
    if "failed" not in rf:
        Vf, Mf, _ = closure.material_sums(pf, fidx, nx * ny)
        err_p = closure.mixed_errors(pp, idx, (Vf, Mf), cells)
        err_l = closure.mixed_errors(pl, idx, (Vf, Mf), cells)
        err_v = closure.mixed_errors(pv, idx, (Vf, Mf), cells)
        cd_p = closure.cell_density_error(pp, idx, (Vf, Mf), cells)
        cd_l = closure.cell_density_error(pl, idx, (Vf, Mf), cells)
    # the literal sinusoidal case under the plain closure
    dk, fr = configs.sod_interface(nx, ny, time_end=0.2)
    pq = Problem.from_deck(dk, material_fraction=fr)
    sq = Solver(pq, fp_mode=fp)
    ierr_q, _ = sq.run(max_steps=20000, history=False)
    literal = {"nel": pq.nel, "mixed_cells": pq.sizes.nmx, "ierr": ierr_q,
               "stopped_at_time": pq.timestep.time, "steps": pq.timestep.nstep,
               "message": sq.error.message.strip() if ierr_q else ""}
    sq.close()
    net.close()
    hbm_peak, peak_kind = load_peaks()
    value = rl["rate"]
    achieved = value * B_LAG / 1e9
    names = ("vol_fraction_abs", "rho1_rel", "rho2_rel")
    return {"metric": METRIC, "what": "two-material Sod with the learned mixed-cell closure",
            "value": value, "unit": "zone-cycles/s", "n_gpus": 1, "steps": rl["steps"],
            "warmup": W, "ms_per_step": rl["ms"] / max(1, rl["steps"]),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "sod2mat_tilted_%dx%d_learned_closure" % (nx, ny),
                       "nel": pp.nel, "mixed_cells": pp.sizes.nmx, "fp_mode": args.fp,
                       "interface": "planar, tilt %.2f; right state rho = p = %.2f"
                                    % CLOSURE_TEST,
                       "timed": "t = 0 to 0.2, %d steps" % rl["steps"],
                       "network": "10-64-64-2 SiLU, BF16 operands, FP32 accumulation",
                       "training": {"samples": int(len(X)),
                                    "cases": sum(len(c) for _, c in CLOSURE_TRAIN_MESHES),
                                    "mesh": " and ".join("%dx%d" % m for m, _ in
                                                         CLOSURE_TRAIN_MESHES) + ", 4x refined",
                                    "epochs": 100,
                                    "loss_first_last": [float(losses[0]), float(losses[-1])],
                                    "data_s": t1 - t0, "train_s": t2 - t1}},
            "plain_closure": {"value": rp["rate"], "unit": "zone-cycles/s", "ms": rp["ms"],
                              "steps": rp["steps"]},
            "refined_plain": ({"refinement": R, "nel": pf.nel, "ms": rf["ms"],
                               "steps": rf["steps"], "value": rf["rate"], "setup_s": fsetup}
                              if "failed" not in rf else
                              {"refinement": R, "nel": pf.nel, "stopped": rf["failed"],
                               "at_time": rf["time"], "after_steps": rf["steps"]}),
            "speedup_vs_refined_plain": rf["ms"] / rl["ms"] if "failed" not in rf else None,
            "closure_cells": {"seen": rl["closure_cells"], "rejected": rl["closure_rejected"]},
            "volume_only": {"value": rv["rate"], "unit": "zone-cycles/s",
                            "errors_vs_refined": (dict(zip(names, err_v))
                                                  if "failed" not in rf else None),
                            "against_plain": {"interface_shift_cells_max": shift_v,
                                              "mixed_cell_density_l1_rel": l1m_v,
                                              "all_cell_density_l1_rel": l1a_v},
                            "closure_cells": {"seen": rv["closure_cells"],
                                              "rejected": rv["closure_rejected"]},
                            "how": "the materials keep their specific energies: the flow "
                                   "stays the plain closure's, the split between the "
                                   "materials is learned"},
            "errors_vs_refined": ({"plain": dict(zip(names, err_p), cell_density_rel_l1=cd_p),
                                   "learned": dict(zip(names, err_l), cell_density_rel_l1=cd_l),
                                   "how": "mean over the mixed cells at t = 0.2 against the "
                                          "%dx-refined run gathered onto the coarse cells" % R}
                                  if "failed" not in rf else None),
            "against_plain": {"interface_shift_cells_max": shift,
                              "mixed_cell_density_l1_rel": l1_mixed,
                              "all_cell_density_l1_rel": l1_all},
            "literal_sinusoidal_plain": literal,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                         "peak_kind": peak_kind,
                         "note": "algorithmic bytes 724 B per zone-cycle (Lagrangian); the "
                                 "FP64 issue rate, not HBM, bounds the path"},
            "e2e": {"value": pe.nel * ne / (t5 - t4), "unit": "zone-cycles/s",
                    "h2d_bytes_per_step": int(h2d / max(1, ne)),
                    "d2h_bytes_per_step": int(h2d / max(1, ne)),
                    "note": "bl_init from the host arrays + bl_set_closure + %d steps of the "
                            "device loop + full download, wall clock" % ne},
            "gpu_launches": rl["launches"], "clocks": rl["clocks"]}


def run_closure_ensemble(args, torch):
    """Batched two-material tubes with the learned closure (--workload
    closure-ensemble; --size = number of tubes, default 64): seeded tubes of
    nx x nx/10 cells, nx log-uniform in [64, 800], interface tilt uniform in
    [0.1, 0.4], right state rho = p uniform in [0.5, 0.6] (the range the
    plain closure survives), each to t = 0.2.  The network is trained as for
    --workload closure.  Timed with CUDA events, whole runs from t = 0 after
    W warm-up steps and a re-upload of the initial state: the batch with
    the learned closure (bl_run_batch, autotuned), the same tubes one after
    another alone with the learned closure, and alone with the plain
    closure (the plain per-mesh GPU path).  Every tube of the batch is then
    compared with its plain-closure run."""
    import ctypes as ct
    import functools
    from bookleaf_f90_gb300 import BatchSolver, Problem, Solver, abi, closure, configs
    fp = {"exact": abi.FP_EXACT, "fast": abi.FP_FAST, "mixed": abi.FP_MIXED}[args.fp]
    n = args.size or 64
    seed = 20240613
    W = max(1, args.warmup)
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(n):
        nx = int(np.exp(rng.uniform(np.log(64), np.log(800))))
        cases.append((max(10, nx), float(rng.uniform(0.1, 0.4)), float(rng.uniform(0.5, 0.6))))
    t0 = time.perf_counter()
    Xs, Ds = [], []
    for (tx, ty), train_cases in CLOSURE_TRAIN_MESHES:
        for case in train_cases:
            X, D, _ = closure.subcell_samples(functools.partial(_closure_case, case), tx, ty,
                                              fp_mode=fp)
            Xs.append(X)
            Ds.append(D)
    net, norm, losses = closure.train(np.concatenate(Xs), np.concatenate(Ds), epochs=100)
    train_s = time.perf_counter() - t0

    def make(i):
        nx, tilt, st = cases[i]
        deck, frac = configs.sod_interface(nx, max(1, nx // 10), time_end=0.2, amplitude=0.0,
                                           periods=0, tilt=tilt, rho_right=st, p_right=st)
        return Problem.from_deck(deck, material_fraction=frac)

    t0 = time.perf_counter()
    probs = [make(i) for i in range(n)]
    setup_s = time.perf_counter() - t0
    nels = [p.nel for p in probs]
    init = [({fid: a.copy() for fid, a in p.fields.items()}, p.timestep.copy()) for p in probs]

    def restore(p, i):
        for fid, a in init[i][0].items():
            np.copyto(p.fields[fid], a)
        ct.memmove(ct.addressof(p.timestep), ct.addressof(init[i][1]), ct.sizeof(abi.Timestep))

    # ---- batched, learned closure
    b = BatchSolver(probs, fp_mode=fp)
    b.set_closure(net, norm)
    tg, tb, _ = b.autotune()
    ierr, _, _ = b.run(max_steps=W)
    assert ierr == 0, b.error.message
    for i, p in enumerate(probs):
        restore(p, i)
    b.sync_to_device(0)
    c0 = b.closure_stats()
    l0 = b.kernel_launches
    stream = torch.cuda.ExternalStream(b.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record(stream)
        ierr, status, nsteps = b.run(max_steps=40000)
        e1.record(stream)
        e1.synchronize()
    assert ierr == 0 and all(p.timestep.time >= 0.2 for p in probs), b.error.message
    ms_b = e0.elapsed_time(e1)
    b.sync_to_host(0)
    c1 = b.closure_stats()
    launches = b.kernel_launches - l0
    b.close()
    zc = sum(nel * p.timestep.nstep for nel, p in zip(nels, probs))
    value = zc / (ms_b * 1e-3)

    # ---- each tube alone: learned closure, then plain closure
    def alone(i, learned):
        q = make(i)
        s = Solver(q, fp_mode=fp)
        if learned:
            s.set_closure(net, norm)
        ierr, _ = s.run(max_steps=W, ts=q.timestep.copy(), history=False)
        assert ierr == 0, s.error.message
        s.sync_to_device(0)
        st = torch.cuda.ExternalStream(s.stream)
        q0 = torch.cuda.Event(enable_timing=True)
        q1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        q0.record(st)
        ierr, _ = s.run(max_steps=40000, history=False)
        q1.record(st)
        q1.synchronize()
        assert ierr == 0, s.error.message
        s.sync_to_host(0)
        s.close()
        return q, q0.elapsed_time(q1)

    ms_l = ms_p = 0.0
    zc_l = zc_p = 0
    shifts, l1m, l1a = [], [], []
    for i in range(n):
        ql, tl = alone(i, True)
        qp, tp = alone(i, False)
        ms_l += tl
        ms_p += tp
        zc_l += ql.nel * ql.timestep.nstep
        zc_p += qp.nel * qp.timestep.nstep
        nx = cases[i][0]
        idx = closure.grid_index(make(i), nx, max(1, nx // 10))
        sh, m1, a1 = closure.against_plain(probs[i], qp, idx, nx, max(1, nx // 10))
        shifts.append(sh)
        l1m.append(m1)
        l1a.append(a1)
    net.close()
    learned_alone = zc_l / (ms_l * 1e-3)
    plain_alone = zc_p / (ms_p * 1e-3)
    hbm_peak, peak_kind = load_peaks()
    achieved = value * B_LAG / 1e9
    return {"metric": METRIC, "what": "batched two-material tubes with the learned closure "
                                      "vs the plain per-mesh GPU path",
            "value": value, "unit": "zone-cycles/s", "n_gpus": 1, "steps": nsteps,
            "warmup": W, "ms_per_step": ms_b / max(1, nsteps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "closure_ensemble_%d_sod2mat_tilted" % n, "tubes": n,
                       "seed": seed, "nel_total": sum(nels), "nel_min": min(nels),
                       "nel_max": max(nels),
                       "mixed_cells_total": sum(p.sizes.nmx for p in probs),
                       "fp_mode": args.fp, "timed": "t = 0 to 0.2 for every tube",
                       "loop": "bl_run_batch, CUDA graphs of %d steps, node block %d "
                               "(autotuned)" % (tg, tb),
                       "training_s": train_s, "setup_s": setup_s},
            "learned_alone": {"value": learned_alone, "unit": "zone-cycles/s", "ms_total": ms_l},
            "plain_alone": {"value": plain_alone, "unit": "zone-cycles/s", "ms_total": ms_p,
                            "how": "each tube alone through bl_run with the plain closure, "
                                   "CUDA events, times summed"},
            "batched_learned_over_plain_alone": value / plain_alone,
            "batched_learned_over_learned_alone": value / learned_alone,
            "closure_cells": {"seen": c1[0] - c0[0], "rejected": c1[1] - c0[1]},
            "against_plain": {"interface_shift_cells_max": max(shifts),
                              "mixed_cell_density_l1_rel_max": max(l1m),
                              "mixed_cell_density_l1_rel_median": float(np.median(l1m)),
                              "all_cell_density_l1_rel_max": max(l1a)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                         "peak_kind": peak_kind,
                         "note": "algorithmic bytes 724 B per zone-cycle (Lagrangian); the "
                                 "FP64 issue rate, not HBM, bounds the path"},
            "gpu_launches": launches, "clocks": clk.summary()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0,
                    help="timed steps; 0 (default) runs the workload to its end time")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--workload", default="sedov")
    ap.add_argument("--size", type=int, default=0)
    ap.add_argument("--fp", default="fast", choices=["fast", "exact", "mixed"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--refine", type=int, default=0,
                    help="closure workload: refinement of the sub-cell truth (0: 4)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    deck, wname, eul = workload_deck(args.workload, args.size)
    bytes_zc = B_EUL if eul else B_LAG

    if args.impl == "reference":
        # The reference's CPU implementation of the path on the host cores.
        # No Fortran compiler exists on either machine, so the reference
        # itself cannot be built; its C restatement (oracle/, -O2, no FMA
        # contraction) stands in.  One independent replica per host core,
        # as the reference's MPI ranks each run the serial loop over their
        # partition.  Under torchrun only rank 0 runs.
        if rank != 0:
            return
        if deck is None:
            why = ("the ensemble is measured against the plain per-mesh GPU path"
                   if args.workload in ("ensemble", "closure-ensemble") else
                   "the reference has no learned closure; its plain closure is timed and "
                   "judged on the GPU beside it")
            print(json.dumps({"impl": "reference", "unavailable":
                              why + "; the CPU arm runs single meshes (--workload sedov|sod|noh)"}))
            return
        from bookleaf_f90_gb300 import Problem
        nel = Problem.from_deck(deck).nel
        cores = os.cpu_count() or 1
        # --steps K: the same K steps from t = 0 as the GPU arm, unless
        # that would take more than about 150 s of CPU time per core (at the
        # restatement's ~3M zone-cycles/s on one core); --steps 0: a
        # sample of about 20 s per core
        req = args.steps
        steps = min(req, max(2, int(150.0 * 3.0e6 / nel))) if req > 0 else 0
        rate, steps, t = cpu_baseline(deck, nel, target_s=20.0, cores=cores, steps=steps,
                                      warmup=min(args.warmup, 1))
        line = {"impl": "reference", "metric": METRIC, "value": rate,
                "unit": "zone-cycles/s", "n_gpus": args.gpus, "steps": steps,
                "warmup": args.warmup, "higher_is_better": True, "dtype": "f64",
                "data": "synthetic", "config": {"workload": wname, "nel": nel},
                "cpu_baseline": {"value": rate, "unit": "zone-cycles/s", "cores": cores,
                                 "kind": "port",
                                 "sample": "the first %d steps of %s from t = 0 on each of %d "
                                           "cores (independent replicas of the serial CPU "
                                           "restatement, -O2 -ffp-contract=off), slowest %.1f s%s"
                                           % (steps, wname, cores, t,
                                              "" if req <= 0 or steps == req else
                                              "; %d requested, capped to bound the run" % req)},
                "e2e": {"value": rate, "unit": "zone-cycles/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
        torch.cuda.set_device(local)
    else:
        torch.cuda.set_device(0)
    from bookleaf_f90_gb300 import Problem, Solver, abi
    from bookleaf_f90_gb300 import build as blbuild
    from bookleaf_f90_gb300.replicas import job_rate
    blbuild.build()
    if args.workload in ("ensemble", "closure", "closure-ensemble"):
        if args.workload == "ensemble":
            line = run_ensemble(args, torch, rank, world)   # every rank its share
            if rank == 0:
                print(json.dumps(line))
        elif rank == 0:
            run = {"closure": run_closure, "closure-ensemble": run_closure_ensemble}[args.workload]
            print(json.dumps(run(args, torch)))
        if world > 1:
            dist.destroy_process_group()
        return

    base = Problem.from_deck(deck)
    nel = base.nel
    fp = {"exact": abi.FP_EXACT, "fast": abi.FP_FAST, "mixed": abi.FP_MIXED}[args.fp]

    # ---------------- value: device-resident time loop ---------------------
    # W warm-up steps, at least one whole graph of the device loop (16
    # steps: its capture and instantiation, a host-side cost paid once per
    # context, then falls outside the timed region), then the initial state
    # is uploaded again and the timed run starts at t = 0: K steps, or with
    # K = 0 the whole run to time_end (the configuration's own end time).
    p = base.copy()
    s = Solver(p, fp_mode=fp)
    init = {fid: arr.copy() for fid, arr in p.fields.items()}
    ts0 = p.timestep.copy()
    warm = max(16, args.warmup)
    ierr, _ = s.run(max_steps=warm, ts=p.timestep.copy(), history=False)
    assert ierr == 0, s.error.message
    for fid, arr in init.items():
        np.copyto(p.fields[fid], arr)
    s.sync_to_device(0)
    ts = ts0.copy()
    stream = torch.cuda.ExternalStream(s.stream)
    l0 = s.kernel_launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    s.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record(stream)
        ierr, _ = s.run(max_steps=args.steps if args.steps > 0 else 10**9, ts=ts, history=False)
        e1.record(stream)
        e1.synchronize()
    s.synchronize()
    torch.cuda.synchronize()
    assert ierr == 0, s.error.message
    nsteps = ts.nstep - ts0.nstep
    t_end = ts.time
    ms = e0.elapsed_time(e1)
    launches = s.kernel_launches - l0
    value, t_max, _ = job_rate(ms, nel * nsteps, device="cuda")
    p.timestep = ts

    # ---------------- per-kernel durations at the end-of-run state --------
    # 16 more steps at the state the run left, the four kernels of each
    # queued back to back on the library's stream with CUDA events between
    # them (no host copies): the mean duration of each kernel.  The profiler
    # range brackets these launches only, so that an ncu capture with
    # --profile-from-start off sees the same launches.
    torch.cuda.profiler.start()
    ierr_k, kms = s.time_step_kernels(16, p.timestep.copy())
    torch.cuda.profiler.stop()
    assert ierr_k == 0, s.error.message
    k_ms = kms[0]
    lag_ms = kms[1] + kms[2] + kms[3]
    hbm_peak, peak_kind = load_peaks()
    achieved = B_GETDT * nel / (k_ms * 1e-3) / 1e9
    prof = load_profile()
    # the capture's figures hold for the FP64 (fast) build on the default
    # workload, where they were taken; elsewhere the line reports none
    if prof and (args.fp != "fast" or not wname.startswith("sedov_512x512_lagrangian")):
        prof = None
    traffic = (prof["dram_bytes_per_launch"] * nel / prof["nel"]) if prof else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "traffic": traffic,
            "traffic_unit": "bytes per launch, from profiles/k_getdt_current.json (ncu, "
                            "dram__bytes_read.sum + dram__bytes_write.sum%s)"
                            % ("" if not prof or prof["nel"] == nel else
                               ", scaled from %d zones" % prof["nel"]),
            "kernel": "k_getdt",
            "peak_kind": peak_kind, "kernel_ms": k_ms,
            "note": "the FP64 issue rate, not HBM, bounds this path; see fp64",
            "lagstep_ms": lag_ms,
            "kernels_ms": {"k_getdt": kms[0], "k_lag_force": kms[1], "k_lag_accel": kms[2],
                           "k_lag_state": kms[3],
                           "how": "mean of 16 steps after the timed run, CUDA events between "
                                  "the kernels on the library's stream"}}
    step_bytes = bytes_zc * nel
    from bookleaf_f90_gb300 import _lib
    rates = _lib.fp64_rates()
    ipz = prof["fp64_pipe_instr_per_zone"] if prof else None
    fp64_ach = ipz * nel / (k_ms * 1e-3) / 1e9 if ipz else None
    fp64 = {"bound": "fp64", "kernel": "k_getdt", "unit": "G FP64-pipe instr/s",
            "achieved": fp64_ach, "peak": rates["dfma"],
            "frac": fp64_ach / rates["dfma"] if ipz else None,
            "peak_kind": "measured live (DFMA issue loop, bl_fp64_rates)",
            "instr_per_zone": ipz,
            "instr_source": "profiles/k_getdt_current.json: %s" % (
                prof["how"] if prof else
                "not applicable: the capture is of the FP64 (fast) build on Sedov 512x512"),
            "rates_gops": rates,
            "step_ms": t_max / max(1, nsteps),
            "hbm_frac_whole_step": (step_bytes * nsteps / (t_max * 1e-3) / 1e9) / hbm_peak}
    s.close()

    # ---------------- e2e through the C-ABI with host buffers --------------
    e2e = None
    if not args.no_e2e:
        pe = base.copy()
        # pin the host arrays so the uploads are DMA transfers
        for fid, arr in list(pe.fields.items()):
            pin = torch.empty(arr.shape, dtype=torch.float64 if arr.dtype.kind == "f" else torch.int32,
                              pin_memory=True).numpy()
            pin[...] = arr
            pe.fields[fid] = pin
        h2d = sum(a.nbytes for a in pe.fields.values())
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        se = Solver(pe, fp_mode=fp)
        ts = pe.timestep
        n_e = 0
        while (n_e < args.steps) if args.steps > 0 else (ts.time < pe.config.time_end):
            assert se.step(ts) == 0, se.error.message
            n_e += 1
        se.sync_to_host(0)
        t1 = time.perf_counter()
        d2h = sum(pe.fields[f].nbytes for f in (abi.ELDENSITY, abi.ELENERGY, abi.ELPRESSURE,
                                                abi.ELCS2, abi.ELVOLUME, abi.A1, abi.A2, abi.A3,
                                                abi.B1, abi.B2, abi.B3, abi.CNWT, abi.CNX, abi.CNY,
                                                abi.CNVISCX, abi.CNVISCY, abi.ELVISC, abi.ELMASS,
                                                abi.CNMASS, abi.NDX, abi.NDY, abi.NDU, abi.NDV)
                  if f in pe.fields)
        e2e_val, _, _ = job_rate((t1 - t0) * 1e3, nel * n_e, device="cuda")
        e2e = {"value": e2e_val, "unit": "zone-cycles/s",
               "h2d_bytes_per_step": int(h2d / n_e) + 2 * 64,
               "d2h_bytes_per_step": int(d2h / n_e) + 3 * 64,
               "note": "bl_init upload of every registered host array + %d per-call steps "
                       "(getdt, lagstep%s; each call uploads the 64-byte step header when the "
                       "host changed it and downloads it) + full state download, host pinned. "
                       "The state stays resident between calls as the reference's dataAPI "
                       "arrays do, so the per-step byte counts are the init upload and the "
                       "final download divided by the %d steps plus the headers"
                       % (n_e, ", alestep" if eul else "", n_e)}
        se.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, steps, t = cpu_baseline(deck, nel, target_s=12.0, cores=1)
        cpu = {"value": rate, "unit": "zone-cycles/s", "cores": 1, "kind": "port",
               "sample": "the first %d steps of %s from t=0 on one core (serial CPU "
                         "restatement, -O2 -ffp-contract=off), %.1f s" % (steps, wname, t)}

    if rank == 0:
        line = {"metric": METRIC, "value": value,
                "unit": "zone-cycles/s", "n_gpus": world, "steps": nsteps,
                "warmup": warm, "ms_per_step": t_max / max(1, nsteps),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": wname, "nel": nel, "fp_mode": args.fp,
                           "replicas": world, "l2": "working set %.0f MB > 129 MB L2, no flush"
                                                     % (step_bytes / 1e6),
                           "timed": "%d steps from t=0 to t=%.4g" % (nsteps, t_end),
                           "loop": "bl_run device time loop, CUDA graphs of 16 steps"},
                "roofline": roof, "fp64": fp64, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches, "clocks": clk.summary()}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
