"""ctypes binding of the reference's own fast-SDF GPU code -- TEST INFRASTRUCTURE ONLY.

``oracle/_ref/libref_rast.so`` is oracle/ref_gpu_harness.cu compiled by
oracle/build_ref.sh around the reference's unmodified
native/src/engine/sdf/cuda_rasterizer.cu (RAST), with the reference's own nvcc flags.
It exists only where the staged reference sources and nvcc are present, and it needs a
GPU to run. Only tests/ and bench.py's reference-on-GPU report use this module: it is a
checker and a reported baseline, never the product.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libref_rast.so"

_lib = None


def available() -> bool:
    return LIB_PATH.exists()


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise FileNotFoundError(f"{LIB_PATH} not built (oracle/build_ref.sh needs the staged reference sources)")
        L = C.CDLL(str(LIB_PATH))
        P, I, F, LL = C.c_void_p, C.c_int, C.c_float, C.c_longlong
        L.refgpu_take_log.argtypes = [C.c_char_p, I]
        L.refgpu_take_log.restype = I
        for name in ("refgpu_fast_sdf", "refgpu_compute_mesh_sdf"):
            getattr(L, name).argtypes = [P, I, F, P, P, P, P]
            getattr(L, name).restype = I
        L.refgpu_splat.argtypes = [P, I, F, P, P, P]
        L.refgpu_splat.restype = I
        for name in ("refgpu_parity", "refgpu_fixup"):
            getattr(L, name).argtypes = [P, I, F, P, P, P]
            getattr(L, name).restype = LL
        for name in ("refgpu_ptd_batch", "refgpu_solid_angle_batch"):
            getattr(L, name).argtypes = [P, P, LL, P]
            getattr(L, name).restype = I
        L.refgpu_sweep.argtypes = [P, P, F, I, I]
        L.refgpu_sweep.restype = I
        L.refgpu_godunov_batch.argtypes = [P, F, LL, P]
        L.refgpu_godunov_batch.restype = I
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _tris(t):
    t = np.ascontiguousarray(np.asarray(t, np.float32).reshape(-1, 12))
    return t, len(t)


def _ivec(v):
    return np.ascontiguousarray(np.asarray(v, np.int32).reshape(3))


def take_log() -> str:
    L = lib()
    n = L.refgpu_take_log(None, 0)
    buf = C.create_string_buffer(n + 1)
    L.refgpu_take_log(buf, n + 1)
    return buf.value.decode(errors="replace")


# RAST:1147-1155: the summary line the fast path logs when it accepts a build.
_OK_RE = re.compile(
    r"Fast SDF path OK: .*? \| eikonal (\d+) rounds .*? fixup (\d+) \| verify (\d+) probes, (\d+) sites, "
    r"(\d+) voxels patched in (\d+) rounds \| far residual (\d+), extra rounds (\d+), safe-clamped (\d+)")


def parse_stats(log: str) -> dict:
    m = _OK_RE.search(log)
    if not m:
        return {}
    keys = ("eikonal_rounds", "fixup_voxels", "probes", "sites", "patched_voxels", "patch_rounds", "far_residual",
            "extra_rounds", "safe_clamped")
    return dict(zip(keys, map(int, m.groups())))


def fast_sdf(tris, h, mn, mx):
    """The reference's fast path forced at any size (RAST:796-1159).
    Returns (accepted, grid or None, the reference's own ms, stats parsed from its log, log)."""
    t, T = _tris(tris)
    mn, mx = _ivec(mn), _ivec(mx)
    N = int(np.prod(mx.astype(np.int64) - mn + 1))
    out = np.empty(N, np.float32)
    ms = C.c_float(0)
    take_log()
    r = lib().refgpu_fast_sdf(_p(t), T, C.c_float(h), _p(mn), _p(mx), _p(out), C.byref(ms))
    log = take_log()
    return r == 1, (out if r == 1 else None), ms.value, parse_stats(log), log


def compute_mesh_sdf(tris, h, mn, mx):
    """CudaRasterizer::compute_mesh_sdf (RAST:1163-1265). Returns (ok, grid, ms, log)."""
    t, T = _tris(tris)
    mn, mx = _ivec(mn), _ivec(mx)
    N = int(np.prod(mx.astype(np.int64) - mn + 1))
    out = np.full(N, np.nan, np.float32)
    ms = C.c_float(0)
    take_log()
    r = lib().refgpu_compute_mesh_sdf(_p(t), T, C.c_float(h), _p(mn), _p(mx), _p(out), C.byref(ms))
    return r == 1, out, ms.value, take_log()


def splat(tris, h, mn, dims):
    """[init] + [A] (RAST:194-268): far sentinel 1e30 outside the band."""
    t, T = _tris(tris)
    dims = _ivec(dims)
    out = np.empty(int(np.prod(dims.astype(np.int64))), np.float32)
    assert lib().refgpu_splat(_p(t), T, C.c_float(h), _p(_ivec(mn)), _p(dims), _p(out)) == 1
    return out


def parity(tris, h, mn, dims):
    """[B] (RAST:279-368) on the supercell CSR of RAST:824-882. Returns (flag, sign u8)."""
    t, T = _tris(tris)
    dims = _ivec(dims)
    sign = np.empty(int(np.prod(dims.astype(np.int64))), np.uint8)
    flag = lib().refgpu_parity(_p(t), T, C.c_float(h), _p(_ivec(mn)), _p(dims), _p(sign))
    assert flag >= -2, "CUDA error in the reference parity driver"
    return int(flag), sign


def fixup(tris, h, mn, dims, sign):
    """[C] (RAST:374-400) on a copy of `sign`. Returns (fixed count, sign)."""
    t, T = _tris(tris)
    dims = _ivec(dims)
    s = np.ascontiguousarray(sign, np.uint8).copy()
    k = lib().refgpu_fixup(_p(t), T, C.c_float(h), _p(_ivec(mn)), _p(dims), _p(s))
    assert k >= 0, "CUDA error in the reference fixup driver"
    return int(k), s


def sweep(grid, dims, h, axis, direction):
    """One directional sweep of gpu_eikonal_fsm_sweep_kernel (RAST:433-513) on a copy of
    `grid`; returns (changed flag, grid). Schedule-independent only when cross-line
    neighbours cannot change during the sweep."""
    g = np.ascontiguousarray(grid, np.float32).copy()
    ch = lib().refgpu_sweep(_p(g), _p(_ivec(dims)), C.c_float(h), int(axis), int(direction))
    assert ch >= 0, "CUDA error in the reference sweep driver"
    return int(ch), g


def ptd_batch(pts, tris9):
    pts = np.ascontiguousarray(pts, np.float32)
    tris9 = np.ascontiguousarray(tris9, np.float32)
    out = np.empty(len(pts), np.float32)
    assert lib().refgpu_ptd_batch(_p(pts), _p(tris9), len(pts), _p(out)) == 1
    return out


def solid_angle_batch(pts, tris9):
    pts = np.ascontiguousarray(pts, np.float32)
    tris9 = np.ascontiguousarray(tris9, np.float32)
    out = np.empty(len(pts), np.float32)
    assert lib().refgpu_solid_angle_batch(_p(pts), _p(tris9), len(pts), _p(out)) == 1
    return out


def godunov_batch(abc, h):
    abc = np.ascontiguousarray(abc, np.float32).reshape(-1, 3)
    out = np.empty(len(abc), np.float32)
    assert lib().refgpu_godunov_batch(_p(abc), C.c_float(h), len(abc), _p(out)) == 1
    return out
