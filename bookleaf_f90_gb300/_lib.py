"""Loader of the in-tree CUDA library (libbookleaf_gb300.so).

There is no CPU fallback: importing works anywhere, but ``load()`` raises
if the library is missing or cannot be loaded, and ``bl_init`` itself fails
when no CUDA device is present.
"""
import ctypes as ct
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_lib", "libbookleaf_gb300.so")

_lib = None


def load(build_if_missing=True):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        if not build_if_missing:
            raise RuntimeError("libbookleaf_gb300.so is not built (run __graft_entry__.build())")
        from . import build
        build.build()
    L = ct.CDLL(LIB)
    P = ct.POINTER
    vp = ct.c_void_p
    L.bl_init.argtypes = [P(vp), P(abi.Sizes), P(abi.Config), vp, ct.c_int, P(abi.Error)]
    L.bl_init.restype = ct.c_int
    L.bl_finalize.argtypes = [vp]
    L.bl_finalize.restype = ct.c_int
    for nm in ("bl_getdt", "bl_lagstep", "bl_alestep"):
        f = getattr(L, nm)
        f.argtypes = [vp, P(abi.Timestep), P(abi.Error)]
        f.restype = ct.c_int
    L.bl_run.argtypes = [vp, P(abi.Timestep), ct.c_int, vp, P(ct.c_int), P(abi.Error)]
    L.bl_run.restype = ct.c_int
    L.bl_sync_to_host.argtypes = [vp, ct.c_int]
    L.bl_sync_to_host.restype = ct.c_int
    L.bl_sync_to_device.argtypes = [vp, ct.c_int]
    L.bl_sync_to_device.restype = ct.c_int
    L.bl_synchronize.argtypes = [vp]
    L.bl_synchronize.restype = ct.c_int
    L.bl_stream.argtypes = [vp]
    L.bl_stream.restype = vp
    L.bl_kernel_launches.argtypes = [vp]
    L.bl_kernel_launches.restype = ct.c_longlong
    L.bl_version.restype = ct.c_char_p
    L.bl_selftest_fp64.argtypes = [ct.c_int, ct.c_longlong, ct.c_ulonglong, P(ct.c_longlong),
                                   P(ct.c_double), P(ct.c_double)]
    L.bl_selftest_fp64.restype = ct.c_int
    L.bl_fp64_rates.argtypes = [P(ct.c_double), ct.c_int]
    L.bl_time_step_kernels.argtypes = [vp, P(abi.Timestep), ct.c_int, P(ct.c_double), ct.c_int,
                                       P(abi.Error)]
    L.bl_time_step_kernels.restype = ct.c_int
    L.bl_init_batch.argtypes = [P(vp), ct.c_int, vp, vp, vp, ct.c_int, P(abi.Error)]
    L.bl_init_batch.restype = ct.c_int
    L.bl_run_batch.argtypes = [vp, vp, ct.c_int, P(ct.c_int), P(ct.c_int), P(abi.Error)]
    L.bl_run_batch.restype = ct.c_int
    L.bl_batch_size.argtypes = [vp]
    L.bl_batch_size.restype = ct.c_int
    L.bl_autotune_batch.argtypes = [vp, vp, P(ct.c_int), P(ct.c_int), P(ct.c_double), ct.c_int,
                                    P(abi.Error)]
    L.bl_autotune_batch.restype = ct.c_int
    L.bl_mlp_create.argtypes = [P(vp), vp]
    L.bl_mlp_create.restype = ct.c_int
    L.bl_mlp_destroy.argtypes = [vp]
    L.bl_mlp_destroy.restype = ct.c_int
    L.bl_mlp_params.argtypes = [vp, vp]
    L.bl_mlp_params.restype = ct.c_int
    L.bl_mlp_predict.argtypes = [vp, vp, ct.c_int, vp]
    L.bl_mlp_predict.restype = ct.c_int
    L.bl_mlp_gradient.argtypes = [vp, vp, vp, ct.c_int, vp, P(ct.c_float)]
    L.bl_mlp_gradient.restype = ct.c_int
    L.bl_mlp_train.argtypes = [vp, vp, vp, ct.c_int, ct.c_int, ct.c_int, ct.c_float,
                               ct.c_ulonglong, vp]
    L.bl_mlp_train.restype = ct.c_int
    L.bl_set_closure.argtypes = [vp, vp, vp, ct.c_int, P(abi.Error)]
    L.bl_set_closure.restype = ct.c_int
    L.bl_closure_stats.argtypes = [vp, P(ct.c_ulonglong), P(ct.c_ulonglong)]
    L.bl_closure_stats.restype = ct.c_int
    L.bl_fp64_rates.restype = ct.c_int
    L.bl_shortprint.argtypes = [vp, ct.c_int, P(ct.c_double), ct.c_int, P(abi.Error)]
    L.bl_shortprint.restype = ct.c_int
    L.bl_check_sod.argtypes = [vp, ct.c_double, P(ct.c_double), P(ct.c_double), P(abi.Error)]
    L.bl_check_sod.restype = ct.c_int
    L.bl_abi_sizes.argtypes = [P(ct.c_int), ct.c_int]
    L.bl_abi_sizes.restype = ct.c_int
    _lib = L
    return L


# Every exported entry point include/bookleaf_gb300.h declares.
EXPORTS = ("bl_init", "bl_finalize", "bl_getdt", "bl_lagstep", "bl_alestep", "bl_run",
           "bl_sync_to_host", "bl_sync_to_device", "bl_synchronize", "bl_stream",
           "bl_kernel_launches", "bl_version", "bl_getdt_noalloc", "bl_selftest_fp64",
           "bl_fp64_rates", "bl_shortprint", "bl_check_sod", "bl_time_step_kernels",
           "bl_init_batch", "bl_run_batch", "bl_batch_size", "bl_autotune_batch",
           "bl_mlp_create", "bl_mlp_destroy", "bl_mlp_params", "bl_mlp_predict",
           "bl_mlp_gradient", "bl_mlp_train", "bl_set_closure", "bl_closure_stats")


def fp64_rates():
    """Measured issue rates on the current device, G operations/s: FP64
    FMA, hardware and integer-pipe divide, square root and multiply."""
    L = load()
    out = (ct.c_double * 7)()
    if L.bl_fp64_rates(out, 7) != 0:
        raise RuntimeError("bl_fp64_rates failed")
    return {"dfma": out[0], "ddiv_hw": out[1], "ddiv_int": out[2], "dsqrt_hw": out[3],
            "dsqrt_int": out[4], "dmul_hw": out[5], "dmul_int": out[6]}
