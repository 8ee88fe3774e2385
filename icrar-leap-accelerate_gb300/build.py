"""Build the GB300 LEAP calibration library in-tree.

Compiles every CUDA translation unit for sm_103a only and the C++ host code
with g++, in parallel, and links ``leap_gb300/_lib/libleap_gb300.so`` plus the
C++ drop-in test driver.  No CMake; the same recipe runs on x86-64 (cross
compile, no GPU) and on the aarch64 GPU hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
CPP = os.path.join(HERE, "cpp")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "leap_gb300", "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libleap_gb300.so")
SYNTH_LIB = os.path.join(OUT_DIR, "libleap_synth.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


CU_SOURCES = ["leap_context.cu", "leap_metadata.cu", "leap_ingest.cu", "leap_calibrate.cu", "leap_adjoint.cu",
              "leap_noalloc.cu"]
CC_SOURCES = ["host_math.cc"]
CPP_SOURCES = ["icrar/calibration.cc", "icrar/MeasurementSet.cc", "icrar/MetaData.cc",
               "icrar/GpuLeapCalibrator.cc", "icrar/LeapCalibratorFactory.cc", "icrar/compute_implementation.cc"]


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = []
    for base in (CSRC, CPP, INCLUDE):
        for dirpath, _, files in os.walk(base):
            hs += [os.path.join(dirpath, f) for f in files if f.endswith((".h", ".cuh", ".hpp"))]
    return hs


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", INCLUDE, "-I", CSRC, "-I", CPP]
    headers = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src.replace("/", "_") + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-warn-spills", *inc, "-c", s, "-o", o])
    cuda_inc = os.path.join(_cuda_home(), "include")
    for src in CC_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src.replace("/", "_") + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", *inc, "-I", cuda_inc,
                         "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CPP, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(OBJ_DIR, src.replace("/", "_") + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-Wall", *inc, "-c", s, "-o", o])
    synth_src = os.path.join(CSRC, "synth_vis.cu")
    synth_obj = os.path.join(OBJ_DIR, "synth_vis.cu.o")
    if force or _newer(synth_obj, [synth_src] + headers):
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *inc, "-c", synth_src,
                     "-o", synth_obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    if force or _newer(SYNTH_LIB, [synth_obj]):
        _run([nvcc, *ARCH, "-shared", "-o", SYNTH_LIB, synth_obj, "-lcudart"])
    tools = []
    for name in ("leap_calibrate_driver", "leap_dropin_bench"):
        src = os.path.join(CPP, "tools", name + ".cc")
        exe = os.path.join(OUT_DIR, name)
        if os.path.exists(src) and (force or _newer(exe, [src, LIB] + headers)):
            tools.append(["g++", "-O2", "-std=c++17", *inc, src, "-o", exe, "-L", OUT_DIR, "-lleap_gb300",
                          "-Wl,-rpath,$ORIGIN"])
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, tools))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
