"""The C-ABI library builds, loads and exports every entry point the header
declares; host-side argument checks work without a GPU.  CPU only."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from ajisai_render_gb300 import _lib, build
    build.build()
    return _lib.load()


def declared_symbols():
    text = (ROOT / "include" / "ajisai_gpu.h").read_text()
    return sorted(set(re.findall(r"AJG_API\s+[\w\s\*]+?\b(ajg_\w+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_symbols()
    for n in ("ajg_create_context", "ajg_scene_create", "ajg_trace_closest",
              "ajg_trace_any", "ajg_render", "ajg_bsdf_query", "ajg_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    for n in declared_symbols():
        assert hasattr(lib, n), n


def test_exports_nothing_else():
    import subprocess
    from ajisai_render_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)],
                         capture_output=True, text=True).stdout
    exported = sorted({l.split()[-1] for l in out.splitlines() if " T " in l})
    assert exported == declared_symbols()


def test_struct_layouts_match_header(lib):
    from ajisai_render_gb300 import _lib
    assert C.sizeof(_lib.Material) == 64
    assert C.sizeof(_lib.Light) == 48
    assert C.sizeof(_lib.Camera) == 144
    assert C.sizeof(_lib.MeshDesc) == 40
    assert C.sizeof(_lib.RenderParams) == 32
    assert C.sizeof(_lib.Emitter) == 32
    assert C.sizeof(_lib.SppmParams) == 40


def test_null_arguments_are_rejected_without_a_gpu(lib):
    assert lib.ajg_abi_version() == 1
    assert lib.ajg_create_context(None, None) == 1          # AJG_ERR_INVALID
    assert b"NULL" in lib.ajg_last_error(None)
    assert lib.ajg_trace_closest(None, None, 0, None) == 1
    assert lib.ajg_render(None, None, None, None) == 1
    assert lib.ajg_scene_release(None) == 1


def test_serving_entry_points_reject_null_arguments(lib):
    """The request loop's entry points check their arguments before they
    touch a device."""
    from ajisai_render_gb300 import _lib
    st = _lib.JobStatus()
    jid = C.c_uint64()
    assert lib.ajg_submit(None, None, C.byref(jid)) == 1
    assert lib.ajg_poll(None, 1, C.byref(st)) == 1
    assert lib.ajg_wait(None, 1, 0, C.byref(st)) == 1
    assert lib.ajg_job_read(None, 1, None, C.byref(st)) == 1
    assert lib.ajg_cancel(None, 1) == 1
    assert lib.ajg_job_release(None, 1) == 1
    assert lib.ajg_render_batch(None, None, 0, None) == 1
    assert lib.ajg_serve_configure(None, None) == 1
    assert lib.ajg_serve_get_stats(None, None) == 1
    assert lib.ajg_image_rmse(None, None, 0, None, 0, 0, 0, None, None) == 1


def test_serving_structs_match_header(lib):
    from ajisai_render_gb300 import _lib
    assert C.sizeof(_lib.JobDesc) == 8 + 144 + 32 + 16 + 8 + 16
    assert C.sizeof(_lib.JobStatus) == 24 + 32
    assert C.sizeof(_lib.ServeOpts) == 16
    assert C.sizeof(_lib.ServeStats) == 88
    assert C.sizeof(_lib.SceneInfo) == 56


def test_context_creation_reports_missing_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = lib.ajg_create_context(None, C.byref(h))
    assert rc == 2 and not h.value                            # AJG_ERR_CUDA
    assert lib.ajg_last_error(None)


def test_film_takes_a_caller_owned_buffer():
    from ajisai_render_gb300 import api
    buf = np.zeros((3, 5, 4), np.float32)
    f = api.Film(5, 3, rgbw=buf)
    assert f.rgbw is buf
    buf[1, 2] = (2.0, 4.0, 6.0, 2.0)
    assert np.allclose(f.image()[1, 2], (1.0, 2.0, 3.0))
    assert api.Film(5, 3).rgbw.shape == (3, 5, 4)
    for bad in (np.zeros((5, 3, 4), np.float32), np.zeros((3, 5, 4), np.float64),
                np.zeros((3, 5, 8), np.float32)[..., ::2]):
        with pytest.raises(ValueError):
            api.Film(5, 3, rgbw=bad)
