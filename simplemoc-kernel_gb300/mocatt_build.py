"""In-tree build of the native libraries (nvcc + gcc, no cmake, no setup.py).

    libmocatt.so    the C-ABI sweep library (include/moc_attenuate.h), CUDA for sm_103a
    libmocsynth.so  the seeded input generator (include/moc_synth.h), plain C
    libmocpeaks.so  roofline microbenchmarks (L2 gather / reduction, FP32, MUFU, HBM)

Objects are rebuilt only when a source or header is newer. Translation units compile in
parallel. Host code is compiled with -ffp-contract=off so it rounds identically on x86
and Arm.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I" + INCLUDE, "-I" + CSRC,
]
CU_SOURCES = ["moc_api.cu", "moc_sweep.cu", "moc_static.cu", "moc_adjoint.cu",
              "moc_batch.cu", "moc_split.cu", "moc_trace.cu", "moc_transport.cu"]
HOST_C_SOURCES = ["trackfile.c"]
# Per-file flags: the track walk rounds every FP64 operation on its own, as the C oracle
# compiled with -ffp-contract=off does, so its descriptors match the oracle's bit for bit.
EXTRA_FLAGS = {"moc_trace.cu": ["-fmad=false"], "moc_transport.cu": ["-fmad=false"]}

LIB = os.path.join(BUILD, "libmocatt.so")
SYNTH_LIB = os.path.join(BUILD, "libmocsynth.so")
PEAKS_LIB = os.path.join(BUILD, "libmocpeaks.so")
DRIVER = os.path.join(BUILD, "mocatt_run")  # C host program (host/moc_driver.c)


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmocatt.so")


def _headers() -> list[str]:
    out = []
    for d in (CSRC, INCLUDE):
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh"))]
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n"
                           f"{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)


def build(verbose: bool = False) -> dict:
    """Build both libraries; returns their paths."""
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + NVCC_FLAGS + EXTRA_FLAGS.get(src, []) + ["-c", s, "-o", o])
    # host-only C of the library (the track file format)
    for src in HOST_C_SOURCES:
        c = os.path.join(HOST, src)
        o = os.path.join(BUILD, src.replace(".c", ".o"))
        objs.append(o)
        if _stale(o, [c] + hdrs):
            jobs.append(["gcc", "-std=gnu99", "-O2", "-ffp-contract=off", "-fPIC",
                         "-I" + INCLUDE, "-c", c, "-o", o])
    synth_src = os.path.join(HOST, "synth.c")
    synth_cmd = None
    if _stale(SYNTH_LIB, [synth_src, os.path.join(INCLUDE, "moc_synth.h")]):
        synth_cmd = ["gcc", "-std=gnu99", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                     "-I" + INCLUDE, synth_src, "-o", SYNTH_LIB, "-lm"]
    peaks_src = os.path.join(CSRC, "moc_peaks.cu")
    if _stale(PEAKS_LIB, [peaks_src]):
        jobs.append([nvcc()] + NVCC_FLAGS + ["-shared", "-cudart", "static", peaks_src,
                                             "-o", PEAKS_LIB])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs) + 1)) as ex:
        futs = [ex.submit(_run, j, verbose) for j in jobs]
        if synth_cmd:
            futs.append(ex.submit(_run, synth_cmd, verbose))
        for f in futs:
            f.result()
    if _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs, verbose)
    driver_src = os.path.join(HOST, "moc_driver.c")
    if _stale(DRIVER, [driver_src, synth_src, LIB] + hdrs):
        _run(["gcc", "-std=gnu99", "-O2", "-ffp-contract=off", "-I" + INCLUDE, driver_src,
              synth_src, "-L" + BUILD, "-lmocatt", "-Wl,-rpath,$ORIGIN", "-lm", "-o", DRIVER],
             verbose)
    return {"libmocatt": LIB, "libmocsynth": SYNTH_LIB, "libmocpeaks": PEAKS_LIB,
            "mocatt_run": DRIVER}


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
