"""Builds the engine's shared library ``libkmcgb300.so`` in-tree with nvcc for sm_103a.

The library is plain C-ABI (include/kmc_gb300.h) with the CUDA runtime linked
statically, so it loads through ctypes (or any FFI) without torch.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libkmcgb300.so")
SOURCES = [os.path.join(CSRC, "kmc_engine.cu"), os.path.join(CSRC, "kmc_run_g16.cu"),
           os.path.join(CSRC, "kmc_solo.cu"), os.path.join(CSRC, "kmc_state.cu"), os.path.join(CSRC, "kmc_otf.cu")]
DEPS = SOURCES + [os.path.join(CSRC, "kmc_device.cuh"), os.path.join(CSRC, "kmc_run.cuh"),
                  os.path.join(CSRC, "kmc_host.h"), os.path.join(CSRC, "kmc_reload.h"), os.path.join(ROOT, "include", "kmc_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in DEPS)


def build(force: bool = False, verbose: bool = False, phase_timing: bool = False, debug: bool = False) -> str:
    """Builds the library (``phase_timing``: a separate libkmcgb300_timing.so with the
    step kernel's per-phase cycle accounting compiled in; ``debug``: a separate
    libkmcgb300_debug.so whose kernels check every table and lattice index they compute
    from table contents, KMC_DEBUG).  Translation units compile in parallel, then link
    into one shared object."""
    lib = LIB.replace(".so", "_timing.so") if phase_timing else LIB.replace(".so", "_debug.so") if debug else LIB
    if not force and not phase_timing and not debug and not needs_build():
        return LIB
    flags = [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include")]
    if verbose:
        flags.insert(0, "-Xptxas=-v")
    if phase_timing:
        flags.insert(0, "-DKMC_PHASE_TIMING")
    if debug:
        flags.insert(0, "-DKMC_DEBUG")
    with tempfile.TemporaryDirectory(prefix="kmcgb300_") as tmpdir:
        objs, procs = [], []
        for src in SOURCES:
            obj = os.path.join(tmpdir, os.path.basename(src) + ".o")
            objs.append(obj)
            procs.append(subprocess.Popen([nvcc(), *flags, "-c", "-o", obj, src]))
        codes = [pr.wait() for pr in procs]
        if any(codes):
            raise subprocess.CalledProcessError(max(codes), "nvcc -c")
        tmp = lib + ".tmp%d" % os.getpid()
        subprocess.check_call([nvcc(), *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    import sys
    build(force=True, verbose="-v" in sys.argv)
    print(LIB)
