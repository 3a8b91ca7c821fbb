"""Build recipe for the oracle (test infrastructure only).

Compiles ``ajg_oracle.cpp`` into ``oracle/_build/libajg_oracle.so`` with
``-ffp-contract=off`` so that no multiply-add is fused (the reference is
compiled for baseline x86-64, which has no FMA; aarch64 would otherwise fuse).

When the reference sources are present (only in the development container),
``build_ref()`` also compiles the reference's own hot-path translation units
plus ``ref_harness/harness.cpp`` into ``oracle/_ref/libajref.so``; that
library only generates the golden fixtures under ``tests/golden``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_SO = BUILD / "libajg_oracle.so"
REF_SO = REF_OUT / "libajref.so"
# Where the reference's sources are mounted (read-only) in the development
# container; AJG_REFERENCE_ROOT points the recipe elsewhere.  Absent on the
# GPU hosts, where only the restatement is built.
REFERENCE_ROOT = Path(os.environ.get("AJG_REFERENCE_ROOT", "/root/reference"))

CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off",
            "-fno-fast-math", "-pthread"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("command failed: " + " ".join(map(str, cmd)))


def _stale(out: Path, srcs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in srcs)


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "ajg_oracle.cpp", HERE / "ajg_oracle.h", HERE / "counter_rng.h"]
    if force or _stale(ORACLE_SO, srcs):
        BUILD.mkdir(parents=True, exist_ok=True)
        tmp = ORACLE_SO.with_suffix(".so.tmp")
        _run(["g++", *CXXFLAGS, "-shared", str(srcs[0]), "-o", str(tmp)])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


# The reference translation units on the PT-MIS / PLOC path that compile
# without their third-party dependencies (Embree, yaml-cpp, spdlog, stb).
REF_TUS = [
    "ajisai/core/aggregate/ploc_aggregate.cpp",
    "ajisai/core/renderer/pt.cpp",
    "ajisai/core/renderer/sppm.cpp",
    "ajisai/core/material/disney.cpp",
    "ajisai/core/material/diffuse.cpp",
    "ajisai/core/material/mirror.cpp",
    "ajisai/core/material/glass.cpp",
    "ajisai/core/material/metal.cpp",
    "ajisai/core/material/plastic.cpp",
    "ajisai/core/material/null.cpp",
    "ajisai/core/material/fresnel.cpp",
    "ajisai/core/bsdf/microfacet_reflection_component.cpp",
    "ajisai/core/bsdf/plastic_bsdf.cpp",
    "ajisai/core/bsdf/aggregate_bsdf.cpp",
    "ajisai/core/bsdf/bsdf.cpp",
    "ajisai/core/bsdf/diffuse_component.cpp",
    "ajisai/core/camera/thin_lens.cpp",
    "ajisai/core/light/directional_light.cpp",
    "ajisai/core/light/env_light.cpp",
    "ajisai/core/light/area_light.cpp",
    "ajisai/core/film.cpp",
    "ajisai/core/parallel.cpp",
    "ajisai/core/scene/default_scene.cpp",
    "ajisai/core/geometry/quad.cpp",
    "ajisai/core/geometry/cube.cpp",
    "ajisai/core/geometry/two_sided.cpp",
    "ajisai/core/primitive/geometric.cpp",
    "ajisai/core/sampler/random_sampler.cpp",
    "ajisai/core/texture2d/constant2d.cpp",
    "ajisai/core/medium/void_medium.cpp",
    "ajisai/core/filter/box_filter.cpp",
]


def reference_available() -> bool:
    return (REFERENCE_ROOT / "ajisai" / "core" / "renderer" / "pt.cpp").exists()


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference's own sources (unmodified, where they lie) with
    the harness.  Returns None when the reference is not present."""
    if not reference_available():
        return None
    harness = HERE / "ref_harness" / "harness.cpp"
    shim = HERE / "ref_harness" / "shim"
    srcs = [REFERENCE_ROOT / t for t in REF_TUS] + [harness]
    if not force and not _stale(REF_SO, srcs + list(shim.rglob("*.h"))):
        return REF_SO
    REF_OUT.mkdir(parents=True, exist_ok=True)
    objdir = REF_OUT / "obj"
    objdir.mkdir(exist_ok=True)
    # Release flags as the reference builds by default (exec.py:8: CMake
    # Release = -O3 -DNDEBUG); baseline x86-64 has no FMA to contract into.
    # glass.cpp names std::optional without including <optional> (its own
    # build gets it through another header): force-include it.
    flags = ["-O3", "-DNDEBUG", "-std=c++20", "-fPIC", "-ffp-contract=off", "-pthread",
             "-w", "-DAJISAI_BUILD_STATIC", "-include", "optional",
             "-I", str(shim), "-I", str(REFERENCE_ROOT)]
    procs, objs = [], []
    for s in srcs:
        o = objdir / (s.stem + ".o")
        objs.append(o)
        # ploc_aggregate.cpp and thin_lens.cpp are also compiled into the
        # harness translation unit (with private members opened) so the
        # harness can read the built tree and the camera matrices; their own
        # objects are left out of the link.
        procs.append(subprocess.Popen(["g++", *flags, "-c", str(s), "-o", str(o)],
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    for p in procs:
        out, err = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out + err)
            raise RuntimeError("reference compile failed")
    objs = [o for o in objs if o.stem not in ("ploc_aggregate", "thin_lens")]
    _run(["g++", "-shared", "-pthread", *map(str, objs), "-o", str(REF_SO)])
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
