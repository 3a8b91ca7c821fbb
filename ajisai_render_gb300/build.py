"""Build libajisai_gpu.so for sm_103a with nvcc (in-tree, no torch).

    python -m ajisai_render_gb300.build [--force]

Each .cu file compiles in parallel to an object under _build/obj, then one
shared library links them with the static CUDA runtime.  Every file is
compiled with -fmad=false (device) and -ffp-contract=off (host): no
multiply-add is contracted, so the non-transcendental arithmetic matches the
reference compiled for baseline x86-64 bit for bit (a build with
AJG_SHADE_FMA=1 contracts the shading unit's arithmetic only).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
BUILD = HERE / "_build"
LIB = BUILD / "libajisai_gpu.so"
# Tuning builds: AJG_BUILD_TAG=<tag> AJG_EXTRA_NVCC="-DAJG_...=..." writes
# _build/libajisai_gpu_<tag>.so; AJG_LIB=<path> makes the loader use it.
TAG = os.environ.get("AJG_BUILD_TAG", "")
EXTRA = os.environ.get("AJG_EXTRA_NVCC", "").split()
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(CSRC.glob("*.cu"))


def headers():
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


# AJG_SHADE_FMA=1: the shading translation units (integrator.cu: ray
# generation, shading, film; capi.cu: the BSDF and camera-ray query kernels
# that share the shading code) are compiled with multiply-add contraction;
# the traversal units keep -fmad=false either way (bit-exact hits).
SHADE_FMA = os.environ.get("AJG_SHADE_FMA", "0") == "1"
FMA_UNITS = ("integrator.cu", "capi.cu")


def flags(extra=(), fmad=False):
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17",
            "-fmad=true" if fmad else "-fmad=false",
            "--expt-relaxed-constexpr", "-Xcompiler",
            "-fPIC,-ffp-contract=off,-fvisibility=hidden",
            "-I", str(INCLUDE), *extra]


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    srcs = sources()
    lib = BUILD / f"libajisai_gpu_{TAG}.so" if TAG else LIB
    if not force and not _stale(lib, srcs + headers() + [Path(__file__)]):
        return lib
    obj = BUILD / (f"obj_{TAG}" if TAG else "obj")
    obj.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    procs = []
    for s in srcs:
        o = obj / (s.stem + ".o")
        cmd = [cc, *flags(EXTRA, SHADE_FMA and s.name in FMA_UNITS), "-c", str(s),
               "-o", str(o)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((s, o, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                             stderr=subprocess.PIPE, text=True)))
    objs, errs = [], []
    for s, o, p in procs:
        out, err = p.communicate()
        if p.returncode != 0:
            errs.append(f"== {s.name}\n{out}{err}")
        elif verbose and err:
            sys.stderr.write(f"== {s.name}\n{err}")
        objs.append(o)
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    tmp = lib.with_suffix(".so.tmp")
    r = subprocess.run([cc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp),
                        *map(str, objs)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, lib)
    return lib


HOST = HERE / "host"
HOST_LIB = BUILD / "libajisai_host.so"
CLI = BUILD / "ajisai_gpu"
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", str(INCLUDE)]


def build_host(force: bool = False) -> Path:
    """The host side (g++, no CUDA): libajisai_host.so -- scene files and
    image output -- and the ajisai_gpu command line, linked against
    libajisai_gpu.so (run from _build/)."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    lib_srcs = [HOST / f for f in ("yaml_lite.cpp", "obj_lite.cpp", "scene_file.cpp",
                                   "image_out.cpp", "host_capi.cpp")]
    deps = sorted(HOST.glob("*.h")) + sorted(HOST.glob("*.cpp")) + headers() + \
        [Path(__file__)]
    BUILD.mkdir(parents=True, exist_ok=True)
    if force or _stale(HOST_LIB, deps):
        tmp = HOST_LIB.with_suffix(".so.tmp")
        r = subprocess.run([cxx, *HOST_FLAGS, "-shared", "-fvisibility=hidden",
                            "-o", str(tmp), *map(str, lib_srcs)],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host library build failed:\n" + r.stderr)
        os.replace(tmp, HOST_LIB)
    if LIB.exists() and (force or _stale(CLI, deps + [LIB])):
        srcs = [HOST / "cli.cpp"] + [x for x in lib_srcs if x.name != "host_capi.cpp"]
        tmp = CLI.with_suffix(".tmp")
        r = subprocess.run([cxx, *HOST_FLAGS, "-o", str(tmp), *map(str, srcs),
                            "-L", str(BUILD), "-lajisai_gpu",
                            "-Wl,-rpath,$ORIGIN"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("ajisai_gpu build failed:\n" + r.stderr)
        os.replace(tmp, CLI)
    return HOST_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    if not TAG:
        print(build_host(force="--force" in sys.argv))
