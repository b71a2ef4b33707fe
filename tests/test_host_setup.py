"""The C++ host side (bookleaf_f90_gb300/host) builds the same initial state
as the Python set-up harness, bit for bit: control-file reader, LIN1/LIN2
mesh, connectivity, node types, regions/materials/mixed cells, initial
conditions, masses, EoS, spmass.  CPU only (the driver's --dump-setup mode
touches no GPU)."""
import ctypes as ct
import os
import struct
import subprocess

import numpy as np
import pytest

from bookleaf_f90_gb300 import Problem, abi, configs
from bookleaf_f90_gb300 import build as blbuild

import golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HG = configs.sedov(16).replace("cvisc2=0.75\n", "cvisc2=0.75\n kappaall=0.05\n pmeritall=0.3\n")
DTNOT = configs.sod(24, 4).replace(
    "cvisc2=0.75\n", "cvisc2=0.75\n zmidlength(2)=.TRUE.\n zdtnotreg(1)=.TRUE.\n")

DECKS = {
    "sod": configs.sod(40, 6),
    "sod_reference_geometry": configs.sod_reference(50, 5),
    "sedov_bench_small": configs.sedov(24, kappa=0.01, pmerit=0.1),
    "sedov_eulerian": configs.sedov(20, eulerian=True),
    "noh": configs.noh(24),
    "noh_eulerian": configs.noh(24, eulerian=True),
    "sod_multimaterial": configs.sod_multimaterial(40, 10),
    "hourglass_subzonal": HG,
    "dtnotreg_midlength": DTNOT,
    "eos_void": configs.eos_tube("void", 30, 4),
    "eos_tait": configs.eos_tube("tait", 30, 4),
    "eos_jwl": configs.eos_tube("jwl", 30, 4),
}


@pytest.fixture(scope="module")
def exe():
    blbuild.build()
    return blbuild.EXE


def read_dump(path):
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == b"BLSETUP1"
    off = 8
    sizes = abi.Sizes.from_buffer_copy(data, off)
    off += ct.sizeof(abi.Sizes)
    config = abi.Config.from_buffer_copy(data, off)
    off += ct.sizeof(abi.Config)
    ts = abi.Timestep.from_buffer_copy(data, off)
    off += ct.sizeof(abi.Timestep)
    (nf,) = struct.unpack_from("<i", data, off)
    off += 4
    fields = {}
    for _ in range(nf):
        fid, kind, n = struct.unpack_from("<iiq", data, off)
        off += 16
        dt = np.float64 if kind == 0 else np.int32
        a = np.frombuffer(data, dtype=dt, count=n, offset=off).copy()
        off += n * np.dtype(dt).itemsize
        fields[fid] = a
    assert off == len(data)
    return sizes, config, ts, fields


def run_dump(exe, deck_text, tmp_path, name):
    dpath = tmp_path / (name + ".deck")
    dpath.write_text(deck_text)
    out = tmp_path / (name + ".bin")
    r = subprocess.run([exe, "--dump-setup", str(out), str(dpath)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return read_dump(out)


def check_same(p, dump):
    sizes, config, ts, fields = dump
    assert bytes(sizes) == bytes(p.sizes)
    assert bytes(config) == bytes(p.config)
    assert bytes(ts) == bytes(p.timestep)
    assert set(fields) == set(p.fields), (sorted(set(fields) ^ set(p.fields)))
    for fid, a in p.fields.items():
        b = fields[fid]
        a = np.ascontiguousarray(a).reshape(-1)
        assert a.dtype == b.dtype, abi.NAMES[fid]
        assert a.shape == b.shape, abi.NAMES[fid]
        same = (a == b) | (np.isnan(a) & np.isnan(b)) if a.dtype.kind == "f" else (a == b)
        assert same.all(), "%s: first difference at %d" % (abi.NAMES[fid], int(np.argmin(same)))


@pytest.mark.parametrize("name", sorted(DECKS))
def test_cpp_setup_matches_python(exe, tmp_path, name):
    deck = DECKS[name]
    check_same(Problem.from_deck(deck), run_dump(exe, deck, tmp_path, name))


@pytest.mark.parametrize("name", golden.deck_names())
def test_cpp_setup_matches_python_on_reference_decks(exe, tmp_path, name):
    """Every control file of the reference (tests/golden/decks)."""
    deck = golden.deck_text(name)
    try:
        p = Problem.from_deck(deck)
    except ValueError as e:  # a deck the harness does not support
        pytest.skip(str(e))
    check_same(p, run_dump(exe, deck, tmp_path, name))


def test_cpp_rejects_what_the_reference_rejects(exe, tmp_path):
    bad = configs.sod(8, 2).replace("time_start=0.0", "time_start=5.0")
    assert bad != configs.sod(8, 2)
    dpath = tmp_path / "bad.deck"
    dpath.write_text(bad)
    r = subprocess.run([exe, "--dump-setup", str(tmp_path / "x.bin"), str(dpath)],
                       capture_output=True, text=True)
    assert r.returncode == 1
    assert "time_start > time_end" in r.stderr
