"""Write tests/golden/oracle_runs.json: regression fixtures of the CPU
restatement (step count, time, dt, and exact checksums of the final fields)
for small runs of each workload family.  The reference itself ships no
golden vectors, so these pin the restatement against accidental change
rather than against the reference.

    python tests/golden/make_golden.py
"""
import json
import os
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from bookleaf_f90_gb300 import abi, configs  # noqa: E402


def _deck(name):
    with open(os.path.join(HERE, "decks", name)) as f:
        return f.read()


CASES = {
    "sod_lag_40x4": (configs.sod(40, 4), 60),
    "sedov_lag_24": (configs.sedov(24), 60),
    "noh_lag_24": (configs.noh(24), 40),
    "noh_eul_24": (configs.noh(24, eulerian=True), 40),
    "sod_mm_20x4": (configs.sod_multimaterial(20, 4), 40),
    # the other equations of state, the hourglass and sub-zonal pressure
    # forces of the benchmark's settings, the polar mesh of ARC sides, and
    # one of the reference's own control files
    "eos_tait_40x4": (configs.eos_tube("tait", 40, 4), 40),
    "eos_jwl_40x4": (configs.eos_tube("jwl", 40, 4), 40),
    "eos_void_40x4": (configs.eos_tube("void", 40, 4), 40),
    "sedov_hg_sp_24": (configs.sedov(24, kappa=0.01, pmerit=0.1), 60),
    "noh_polar_20x8": (configs.noh_polar(20, 8), 40),
    "deck_sod_mm_lag_small": (_deck("sod_mm_lag_small"), 20),
}


def _bits(a):
    """Exact checksum of a float64 array: the first 16 hex digits of the
    SHA-256 of its little-endian bytes in order, so any change of any bit
    of any element, or of the elements' order, changes it."""
    import hashlib
    import numpy as np
    v = np.ascontiguousarray(a, dtype="<f8")
    return hashlib.sha256(v.tobytes()).hexdigest()[:16]


def summarise(p):
    ts = p.timestep
    out = {"nstep": ts.nstep, "time": struct.unpack("<Q", struct.pack("<d", ts.time))[0],
           "dt": struct.unpack("<Q", struct.pack("<d", ts.dt))[0]}
    for fid in (abi.ELDENSITY, abi.ELENERGY, abi.NDX, abi.NDY, abi.NDU, abi.NDV):
        out[abi.NAMES[fid]] = _bits(p.fields[fid])
    return out


def main():
    from bookleaf_f90_gb300 import Problem
    from oracle.oracle import Oracle
    res = {}
    for name, (deck, steps) in CASES.items():
        p = Problem.from_deck(deck)
        o = Oracle(p)
        ierr, n = o.run(p.timestep, steps)
        assert ierr == 0
        res[name] = summarise(p)
        print(name, res[name]["nstep"])
    with open(os.path.join(HERE, "oracle_runs.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
