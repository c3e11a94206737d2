"""Build recipe of the GB300 engine: nvcc for sm_103a, gcc for the host C.

Produces, in this directory:
  libedmd_gpu.so  C ABI of include/edmd_gpu.h + include/edmd_host.h
  edmd            drop-in command-line driver (host/edmd_main.c), rpath to the .so
and, only with `python build.py probe`, the measurement tool peak_probe
(probe/peak_probe.cu: FP64 issue rate and load latency).

All CUDA is compiled for sm_103a only, with --fmad=false so that no
floating-point multiply-add is contracted (the event arithmetic must round
exactly like the reference compiled with IEEE flags).  Translation units are
compiled in parallel; no cmake.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")

CUDA_SOURCES = ["edmd_engine.cu", "edmd_lane.cu", "edmd_tangent.cu", "edmd_round.cu", "edmd_observe.cu"]
HOST_SOURCES = ["edmd_init.c"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false",
              "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
CC_FLAGS = ["-O2", "-fno-fast-math", "-ffp-contract=off", "-fPIC", "-Wall", "-I" + INCLUDE]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _newer(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run_all(cmds):
    procs = [(subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), c) for c in cmds]
    err = []
    for p, c in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            err.append(" ".join(c) + "\n" + out)
    if err:
        raise RuntimeError("build failed:\n" + "\n".join(err))


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    objs, cmds = [], []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers + [__file__]):
            cmds.append([_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj])
    for s in HOST_SOURCES:
        src = os.path.join(HOST, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers + [__file__]):
            cmds.append(["gcc"] + CC_FLAGS + ["-c", src, "-o", obj])
    _run_all(cmds)
    lib = os.path.join(HERE, "libedmd_gpu.so")
    if _newer(lib, objs):
        _run_all([[_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", lib]
                  + objs + ["-lcudart", "-lpthread", "-lm"]])
    main_src = os.path.join(HOST, "edmd_main.c")
    exe = os.path.join(HERE, "edmd")
    if os.path.exists(main_src) and _newer(exe, [main_src, lib] + headers):
        _run_all([["gcc"] + CC_FLAGS + ["-o", exe, main_src, "-L" + HERE, "-ledmd_gpu",
                   "-Wl,-rpath,$ORIGIN", "-lm"]])
    return lib


def build_probe():
    """The FP64/FP32 issue-rate and load-latency microbenchmark behind the
    engines' FP64 roofline (not part of the library): ./peak_probe."""
    src = os.path.join(HERE, "probe", "peak_probe.cu")
    exe = os.path.join(HERE, "peak_probe")
    if _newer(exe, [src, __file__]):
        _run_all([[_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe, src]])
    return exe


if __name__ == "__main__":
    print(build_probe() if sys.argv[1:] == ["probe"] else build(verbose=True))
    sys.exit(0)
