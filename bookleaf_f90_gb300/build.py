"""Build the sm_103a shared library libbookleaf_gb300.so in-tree.

Eight translation units, compiled in parallel with nvcc:
  bl_kernels.cu  -DBL_NS=fast  --fmad=true   (fused multiply-add and exact
                 -DBL_FAST_ALGEBRA=1          algebraic identities allowed)
  bl_kernels.cu  -DBL_NS=exact --fmad=false  (bit-reproducible path)
  bl_kernels.cu  -DBL_NS=mixed --fmad=true   (the fast build with the limiter
                 -DBL_MIXED=1                 arithmetic in FP32; FP32 divide and
                 -prec-div/-prec-sqrt=false   square root approximate, FP32
                 -ftz=true                    subnormals flushed: FP64 untouched)
  bl_capi.cu                                  (the C-ABI, host code)
  bl_noalloc.cu  --fmad=false                 (allocation-free getdt: the exact
                                              build's k_getdt)
  bl_selftest.cu                              (FP64 self-test and rates)
  bl_diag.cu     --fmad=false                 (short print, Sod check)
  bl_mlp.cu                                   (the closure network, tensor cores)
and linked with the CUDA runtime statically, so the library needs nothing
but the driver at run time.

The C++ host side (host/: control-file reader, mesh generator, initial
state, solver entry points over the C-ABI) is compiled with g++ alongside
(-ffp-contract=off, so its set-up arithmetic is the reference's operation
for operation) and linked into the driver executable _lib/bookleaf_gb300.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUTDIR = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(OUTDIR, "libbookleaf_gb300.so")
EXE = os.path.join(OUTDIR, "bookleaf_gb300")
HOST_SOURCES = ("deck", "mesh", "ic", "problem", "solver", "io", "main")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _sources():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(HOST, f) for f in os.listdir(HOST)]
    deps.append(os.path.join(HERE, "..", "include", "bookleaf_gb300.h"))
    return deps


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUTDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _sources())
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest
            and os.path.exists(EXE) and os.path.getmtime(EXE) >= newest):
        return LIB
    cc = nvcc()
    common = [cc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                            "-Xptxas", "-v" if verbose else "-O3"] + list(extra)
    jobs = [
        (common + ["--fmad=true", "-DBL_NS=fast", "-DBL_FAST_ALGEBRA=1", "-c",
                   os.path.join(CSRC, "bl_kernels.cu"),
                   "-o", os.path.join(BUILD, "k_fast.o")]),
        (common + ["--fmad=false", "-DBL_NS=exact", "-c", os.path.join(CSRC, "bl_kernels.cu"),
                   "-o", os.path.join(BUILD, "k_exact.o")]),
        (common + ["--fmad=true", "-DBL_NS=mixed", "-DBL_FAST_ALGEBRA=1", "-DBL_MIXED=1",
                   "-DBL_GETDT_SPLIT=1",
                   "-ftz=true", "-prec-div=false", "-prec-sqrt=false", "-c",
                   os.path.join(CSRC, "bl_kernels.cu"), "-o", os.path.join(BUILD, "k_mixed.o")]),
        (common + ["-c", os.path.join(CSRC, "bl_capi.cu"), "-o", os.path.join(BUILD, "capi.o")]),
        (common + ["--fmad=false", "-c", os.path.join(CSRC, "bl_noalloc.cu"),
                   "-o", os.path.join(BUILD, "noalloc.o")]),
        (common + ["-c", os.path.join(CSRC, "bl_selftest.cu"), "-o", os.path.join(BUILD, "selftest.o")]),
        (common + ["--fmad=false", "-c", os.path.join(CSRC, "bl_diag.cu"),
                   "-o", os.path.join(BUILD, "diag.o")]),
        (common + ["-c", os.path.join(CSRC, "bl_mlp.cu"), "-o", os.path.join(BUILD, "mlp.o")]),
    ]
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    for name in HOST_SOURCES:
        jobs.append([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                     "-c", os.path.join(HOST, name + ".cpp"), "-o", os.path.join(BUILD, "h_" + name + ".o")])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    logs = []
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        logs.append(out.decode(errors="replace"))
        if p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
            raise RuntimeError("compile failed: " + " ".join(j))
    tmp = LIB + ".%d.tmp" % os.getpid()
    subprocess.check_call([cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp,
                                         os.path.join(BUILD, "k_fast.o"),
                                         os.path.join(BUILD, "k_exact.o"),
                                         os.path.join(BUILD, "k_mixed.o"),
                                         os.path.join(BUILD, "capi.o"),
                                         os.path.join(BUILD, "noalloc.o"),
                                         os.path.join(BUILD, "selftest.o"),
                                         os.path.join(BUILD, "diag.o"),
                                         os.path.join(BUILD, "mlp.o")])
    os.replace(tmp, LIB)
    tmp = EXE + ".%d.tmp" % os.getpid()
    subprocess.check_call([cxx, "-o", tmp] + [os.path.join(BUILD, "h_" + n + ".o") for n in HOST_SOURCES]
                          + ["-L" + OUTDIR, "-lbookleaf_gb300", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, EXE)
    if verbose:
        sys.stdout.write("\n".join(logs))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
