"""The integer-pipe FP64 divide, square root and multiply the kernels use
must equal the hardware operations bit for bit (bl_fp64.cuh, checked on the
device)."""
import ctypes as ct

import pytest

pytestmark = pytest.mark.gpu


def _selftest(op, n, seed):
    from bookleaf_f90_gb300 import _lib
    L = _lib.load()
    bad = ct.c_longlong(-1)
    a = ct.c_double(0)
    b = ct.c_double(0)
    assert L.bl_selftest_fp64(op, n, seed, ct.byref(bad), ct.byref(a), ct.byref(b)) == 0
    return bad.value, a.value, b.value


@pytest.mark.parametrize("seed", [1, 0x5EED, 0xB00C1EAF])
def test_divide_matches_hardware(seed):
    bad, a, b = _selftest(0, 1 << 28, seed)
    assert bad == 0, "first mismatch %r / %r" % (a, b)


@pytest.mark.parametrize("seed", [2, 0xC0FFEE, 0xFEEDFACE])
def test_sqrt_matches_hardware(seed):
    bad, a, _ = _selftest(1, 1 << 28, seed)
    assert bad == 0, "first mismatch sqrt(%r)" % (a,)


@pytest.mark.parametrize("seed", [3, 0xD1CE, 0x7E57AB1E])
def test_multiply_matches_hardware(seed):
    bad, a, b = _selftest(2, 1 << 28, seed)
    assert bad == 0, "first mismatch %r * %r" % (a, b)


def test_integer_pipe_rates_beat_hardware():
    """The reason the kernels use them: on GB300 the integer-pipe divide and
    square root issue faster than the FP64-pipe ones."""
    from bookleaf_f90_gb300 import _lib
    r = _lib.fp64_rates()
    assert r["dfma"] > 100.0, r
    assert r["ddiv_int"] > r["ddiv_hw"], r
    assert r["dsqrt_int"] > r["dsqrt_hw"], r
