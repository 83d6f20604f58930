"""The C-ABI library loads and exports every function include/gbsdf.h declares (CPU:
no compute call is made). Also checks the Python mirror's struct layouts against
the header's sizes."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gbsdf.h"


def declared_functions():
    src = HEADER.read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_\s\*]*?\b(gbsdf_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib_path():
    from gbsdf import _lib

    if not _lib.LIB_PATH.exists():
        from gbsdf import build

        build.build()
    return _lib.LIB_PATH


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("gbsdf_compute_mesh_sdf", "gbsdf_build_from_mesh", "gbsdf_mesh_lattice", "gbsdf_default_options"):
        assert n in names


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(gbsdf_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_binds(lib_path):
    from gbsdf import _lib

    L = _lib.load()
    for n in declared_functions():
        assert hasattr(L, n)
    assert set(_lib.EXPORTS) <= set(declared_functions())
    # every bound entry point has its C signature (ctypes would pass 64-bit pointers and
    # sizes as 32-bit ints otherwise)
    unbound = [n for n in _lib.EXPORTS if getattr(L, n).argtypes is None]
    assert not unbound, unbound
    assert b"sm_103a" in L.gbsdf_version()


def test_struct_layouts():
    from gbsdf import _lib

    assert C.sizeof(_lib.Options) == 64
    # 2 int32 + 10 float + 6 int32 + 11 int64 + 6 int64, escalated, band_err_fp64 (double), band_err_samples,
    # ms_sweeps (float) + sweep_schedule_first (int32)
    assert C.sizeof(_lib.Stats) == 8 + 40 + 24 + 88 + 64 + 8


def test_default_options_and_lattice_need_no_gpu(lib_path):
    import numpy as np

    from gbsdf import _lib, api

    L = _lib.load()
    o = _lib.Options()
    L.gbsdf_default_options(C.byref(o))
    assert o.mode == _lib.MODE_REFERENCE and o.path == _lib.PATH_AUTO and o.device == 0
    # lattice is host arithmetic (cuda_rasterizer.cu:1358-1372)
    v = np.array([[0, 0, 0], [1, 2, 3]], np.float32)
    mn, mx = api.mesh_lattice(v, 0.5)
    assert list(mn) == [-10, -10, -10] and list(mx) == [12, 14, 16]
