"""The C-ABI library: builds, loads, exports every declared entry point, and
its structs match the ctypes mirrors (CPU only: no kernel is launched)."""
import ctypes as ct
import os
import re

import pytest

from bookleaf_f90_gb300 import Problem, abi, configs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bookleaf_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from bookleaf_f90_gb300 import _lib
    return _lib.load()


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void \*|long long|const char \*)\s*(bl_\w+)\(",
                                 text, re.M)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "bl_init" in names and "bl_lagstep" in names
    for n in names:
        assert hasattr(lib, n), n


def test_struct_sizes_match_header(lib):
    out = (ct.c_int * 5)()
    assert lib.bl_abi_sizes(out, 5) == 5
    assert out[0] == ct.sizeof(abi.Sizes)
    assert out[1] == ct.sizeof(abi.Config)
    assert out[2] == ct.sizeof(abi.Timestep)
    assert out[3] == ct.sizeof(abi.Error)
    assert out[4] == ct.sizeof(abi.StepRecord)


def test_version(lib):
    assert b"sm_103a" in lib.bl_version()


def test_init_fails_loudly_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from bookleaf_f90_gb300 import Solver, SolverError
    p = Problem.from_deck(configs.sod(8, 2))
    with pytest.raises(SolverError) as ex:
        Solver(p)
    assert "CUDA" in str(ex.value)


def test_init_rejects_bad_connectivity(lib):
    """A bad node number is refused (on a machine without a GPU the refusal
    is the missing device; the device-side check has its own tests)."""
    p = Problem.from_deck(configs.sod(8, 2))
    p.fields[abi.IELND][3, 1] = p.nnd + 5
    err = abi.Error()
    ctx = ct.c_void_p()
    tab = p.pointer_table()
    ierr = lib.bl_init(ct.byref(ctx), ct.byref(p.sizes), ct.byref(p.config),
                       ct.cast(tab, ct.c_void_p), 0, ct.byref(err))
    assert ierr == abi.FAILURE
    assert "out of range" in err.message or "CUDA" in err.message


def test_closure_entry_points_reject_bad_arguments(lib):
    """bl_set_closure / bl_closure_stats check their arguments before any
    CUDA call: no context, an unknown mode, or a mode without a network."""
    err = abi.Error()
    norm = (ct.c_float * 22)()
    assert lib.bl_set_closure(None, None, None, 0, ct.byref(err)) == abi.FAILURE
    assert "bad argument" in err.message
    assert lib.bl_set_closure(None, None, norm, 3, ct.byref(err)) == abi.FAILURE
    a, b = ct.c_ulonglong(7), ct.c_ulonglong(7)
    assert lib.bl_closure_stats(None, ct.byref(a), ct.byref(b)) == abi.FAILURE
