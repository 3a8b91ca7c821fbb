"""The reference-side adapters (ajisai_render_gb300/adapters: the "pt_gpu"
renderer and the "ploc_gpu" aggregate) compiled against the reference's own
headers (renderer.h:53-59, aggregate.h:32-42) and linked against
libajisai_gpu, with the reference's compiled sources from the oracle
harness.  Without a GPU (this suite runs on the CPU): the triangles they
hand the library are the reference's own MeshView gathering, and both
adapters stop with the library's error message through ajg_last_error, in
the reference's convention (a message, then exit status 1).  Skipped where
the reference's sources are absent."""
import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    from oracle import build as ob
    if not ob.reference_available():
        pytest.skip("the reference's sources are not available here")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the no-device paths do not apply")
    from ajisai_render_gb300 import build as gb
    ref = ob.build_ref()
    gpu = gb.build()
    host = gb.build_host()
    out = tmp_path_factory.mktemp("adapters") / "libadapter_test.so"
    cmd = ["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-w",
           "-DAJISAI_BUILD_STATIC", "-include", "optional",
           "-I", str(ob.HERE / "ref_harness" / "shim"), "-I", str(ob.REFERENCE_ROOT),
           "-I", str(ROOT / "include"),
           str(ROOT / "ajisai_render_gb300" / "adapters" / "gpu_adapters.cpp"),
           str(ROOT / "tests" / "adapter_shim.cpp"),
           str(ref), str(gpu), str(host),
           f"-Wl,-rpath,{ref.parent}:{gpu.parent}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def test_adapters_gather_the_reference_triangles(shim):
    from ajisai_render_gb300 import scenes as S
    from oracle import pyoracle as O
    rs = O.RefScene(S.cornell_box(8, 8))
    lib = C.CDLL(str(shim))
    lib.adapter_gather.restype = C.c_int64
    lib.adapter_gather.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                   C.c_void_p]
    cap = 1000
    tris = np.zeros((cap, 9), np.float32)
    world = np.zeros(6, np.float32)
    ids = np.zeros(cap, np.int64)
    n = lib.adapter_gather(rs.h, tris.ctypes.data, cap, world.ctypes.data,
                           ids.ctypes.data)
    d = rs.dump()
    assert n == d.n_tris == 34
    assert np.array_equal(tris[:n].view(np.uint32), d.tris.view(np.uint32))
    assert np.array_equal(world.view(np.uint32), d.world.view(np.uint32))


def _run(code):
    return subprocess.run([sys.executable, "-c", code], capture_output=True,
                          text=True, timeout=300, cwd=ROOT)


def test_renderer_adapter_reports_the_library_error(shim):
    scene = ROOT / "tests" / "golden" / "scenes" / "cornell_box.yaml"
    r = _run(f"import ctypes as C; C.CDLL({str(shim)!r}).adapter_render("
             f"{str(scene).encode()!r}, 256, 256, 4)")
    assert r.returncode == 1, (r.stdout, r.stderr)
    assert "ajisai_gpu: ajg_create_context failed (2)" in r.stderr, r.stderr


def test_aggregate_adapter_reports_the_library_error(shim):
    code = f"""
import ctypes as C, sys
sys.path.insert(0, {str(ROOT)!r})
from ajisai_render_gb300 import scenes as S
from oracle import pyoracle as O
rs = O.RefScene(S.cornell_box(8, 8))
lib = C.CDLL({str(shim)!r})
lib.adapter_build_aggregate.argtypes = [C.c_void_p, C.c_int64]
lib.adapter_build_aggregate(rs.h, 14)
"""
    r = _run(code)
    assert r.returncode == 1, (r.stdout, r.stderr)
    assert "ajisai_gpu: ajg_create_context failed (2)" in r.stderr, r.stderr
