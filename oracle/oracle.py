"""ctypes binding of the CPU oracle (oracle/sdf_oracle.cpp) -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference arm
import this module. It checks the product; it is never the product.

Every function cites the reference code it restates (paths relative to the
reference project): the fast SDF path in native/src/engine/sdf/cuda_rasterizer.cu
(RAST) and the primitives in native/src/core/math_utils.cuh (MATH).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
SRC = HERE / "sdf_oracle.cpp"
SRCS = [SRC, HERE / "meshio_oracle.cpp"]
REF_LIB_PATH = HERE / "_ref" / "libref_math.so"

# fast-path status codes (orc_fast_stats.status)
OK, INVALID, INT_GUARD, CSR_GUARD, VERIFY_DIVERGED = 0, 1, 2, 3, 4


def build(force: bool = False) -> Path:
    """Compile the oracle with g++ (no FP contraction, so x86 and Arm agree)."""
    if force or not LIB_PATH.exists() or any(LIB_PATH.stat().st_mtime < p.stat().st_mtime for p in SRCS):
        cmd = ["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
               *map(str, SRCS), "-o", str(LIB_PATH)]
        subprocess.check_call(cmd)
    return LIB_PATH


def build_ref(reference_root=None) -> Path | None:
    """Compile the reference's own primitives into oracle/_ref: from the reference tree at
    ``reference_root`` (or the RHIZOME_REFERENCE environment variable) where given, and the
    reference GPU checker from the staged sources wherever they are."""
    env = dict(os.environ)
    if reference_root is not None:
        env["RHIZOME_REFERENCE"] = str(reference_root)
    subprocess.check_call(["bash", str(HERE / "build_ref.sh")], env=env)
    return REF_LIB_PATH if REF_LIB_PATH.exists() else None


class FastParams(C.Structure):
    _fields_ = [("fsm_mode", C.c_int), ("gwn_mode", C.c_int), ("threads", C.c_int),
                ("max_conv_rounds", C.c_int), ("skip_verify", C.c_int), ("signed_parity", C.c_int),
                ("skip_eikonal", C.c_int), ("lazy_winding", C.c_int)]


class FastStats(C.Structure):
    _fields_ = [("status", C.c_int), ("unknown_columns", C.c_int), ("fixup_voxels", C.c_longlong),
                ("eikonal_rounds", C.c_int), ("extra_rounds", C.c_int), ("far_residual", C.c_longlong),
                ("safe_clamped", C.c_longlong), ("probes", C.c_int), ("sites", C.c_int),
                ("patch_rounds", C.c_int), ("patched_voxels", C.c_longlong), ("fp64_rechecks", C.c_longlong),
                ("band_voxels", C.c_longlong),
                ("ms_splat", C.c_double), ("ms_parity", C.c_double), ("ms_fixup", C.c_double),
                ("ms_eikonal", C.c_double), ("ms_verify", C.c_double), ("ms_apply", C.c_double),
                ("ms_total", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        L.orc_point_triangle_distance_sq.restype = C.c_float
        L.orc_triangle_solid_angle.restype = C.c_float
        L.orc_triangle_solid_angle_f64.restype = C.c_double
        L.orc_godunov.restype = C.c_float
        L.orc_godunov.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float]
        L.orc_splat_band.restype = C.c_longlong
        L.orc_parity_signs.restype = C.c_longlong
        L.orc_parity_signs_mode.restype = C.c_longlong
        L.orc_fixup_unknown.restype = C.c_longlong
        L.orc_fsm_sweep.restype = C.c_int
        L.orc_eikonal.restype = C.c_int
        L.orc_verify_patch.restype = C.c_int
        L.orc_fast_sdf.restype = C.c_int
        L.orc_lattice.restype = C.c_int
        L.orc_build_triangles.restype = C.c_longlong
        L.orc_fast_min_voxels.restype = C.c_longlong
        for name in ("orc_splat_band", "orc_parity_signs", "orc_fixup_unknown", "orc_fast_sdf",
                     "orc_legacy_sdf", "orc_gwn_points_f64", "orc_gwn_sign_voxels", "orc_ptd_batch",
                     "orc_solid_angle_batch", "orc_lattice", "orc_build_triangles", "orc_fsm_sweep",
                     "orc_eikonal", "orc_apply_signs", "orc_verify_patch"):
            getattr(L, name).restype = getattr(L, name).restype
        _ = P
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _ivec(v):
    return np.ascontiguousarray(np.asarray(v, np.int32).reshape(3))


def _tris(t):
    t = np.ascontiguousarray(np.asarray(t, np.float32).reshape(-1, 12))
    return t, len(t)


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


# ---- primitives (MATH:43-132) -------------------------------------------------------
def ptd_batch(pts, tris9):
    pts = np.ascontiguousarray(pts, np.float32)
    tris9 = np.ascontiguousarray(tris9, np.float32)
    out = np.empty(len(pts), np.float32)
    lib().orc_ptd_batch(_p(pts), _p(tris9), C.c_longlong(len(pts)), _p(out))
    return out


def solid_angle_batch(pts, tris9):
    pts = np.ascontiguousarray(pts, np.float32)
    tris9 = np.ascontiguousarray(tris9, np.float32)
    out = np.empty(len(pts), np.float32)
    lib().orc_solid_angle_batch(_p(pts), _p(tris9), C.c_longlong(len(pts)), _p(out))
    return out


def godunov(ax, ay, az, h):
    """rhi_eikonal_godunov, RAST:405-425."""
    return lib().orc_godunov(float(ax), float(ay), float(az), float(h))


def gwn_points_f64(tris, pts, threads=None):
    t, T = _tris(tris)
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    out = np.empty(len(pts), np.float64)
    lib().orc_gwn_points_f64(_p(t), C.c_int(T), _p(pts), C.c_longlong(len(pts)), _p(out),
                             C.c_int(threads or default_threads()))
    return out


def gwn_sign_voxels(tris, h, mn, dims, vidx, mode=1, threads=None):
    t, T = _tris(tris)
    vidx = np.ascontiguousarray(vidx, np.int64)
    out = np.empty(len(vidx), np.uint8)
    lib().orc_gwn_sign_voxels(_p(t), C.c_int(T), C.c_float(h), _p(_ivec(mn)), _p(_ivec(dims)), _p(vidx),
                              C.c_longlong(len(vidx)), C.c_int(mode), _p(out), C.c_int(threads or default_threads()))
    return out


# ---- stages ----------------------------------------------------------------------------
def splat_band(tris, h, mn, dims, threads=None):
    """[init]+[A]: sentinel fill and exact band splat (RAST:194-268). Returns (dist, band_count)."""
    t, T = _tris(tris)
    dims = _ivec(dims)
    dist = np.empty(int(np.prod(dims.astype(np.int64))), np.float32)
    n = lib().orc_splat_band(_p(t), C.c_int(T), C.c_float(h), _p(_ivec(mn)), _p(dims), _p(dist),
                             C.c_int(threads or default_threads()))
    return dist, n


def parity_signs(tris, h, mn, dims, threads=None, signed=False):
    """[B]: scanline parity (RAST:279-368, CSR RAST:824-882), or signed crossings
    (winding number along the column) with ``signed``. Returns (sign u8, unknown_columns)."""
    t, T = _tris(tris)
    dims = _ivec(dims)
    sign = np.empty(int(np.prod(dims.astype(np.int64))), np.uint8)
    n = lib().orc_parity_signs_mode(_p(t), C.c_int(T), C.c_float(h), _p(_ivec(mn)), _p(dims), _p(sign),
                                    C.c_int(threads or default_threads()), C.c_int(1 if signed else 0))
    return sign, n


def fixup_unknown(tris, h, mn, dims, sign, dist=None, gwn_mode=1, threads=None):
    """[C]: exact winding for sign==2 voxels (RAST:374-400). In place; returns count.
    ``dist``: the band field (on-surface voxels, |d| <= 1e-5 voxel, count as inside)."""
    t, T = _tris(tris)
    rech = C.c_longlong(0)
    dp = _p(np.ascontiguousarray(dist, np.float32)) if dist is not None else None
    n = lib().orc_fixup_unknown(_p(t), C.c_int(T), C.c_float(h), _p(_ivec(mn)), _p(_ivec(dims)), _p(sign), dp,
                                C.c_int(gwn_mode), C.c_int(threads or default_threads()), C.byref(rech))
    return n


def fsm_sweep(g, dims, h, axis, direction, threads=None):
    """[D]: one directional sweep (RAST:433-513), in place. Returns changed flag."""
    return lib().orc_fsm_sweep(_p(g), _p(_ivec(dims)), C.c_float(h), C.c_int(axis), C.c_int(direction),
                               C.c_int(threads or default_threads()))


def eikonal(g, sign, dims, h, fsm_mode=1, max_conv_rounds=100000, threads=None):
    """[D]/[D2]/[D3]: FSM rounds, audit, clamp (RAST:987-1064), in place."""
    extra = C.c_int(0)
    resid = C.c_longlong(0)
    clamped = C.c_longlong(0)
    r = lib().orc_eikonal(_p(g), _p(sign), _p(_ivec(dims)), C.c_float(h), C.c_int(fsm_mode),
                          C.c_int(max_conv_rounds), C.c_int(threads or default_threads()), C.byref(extra),
                          C.byref(resid), C.byref(clamped))
    return dict(rounds=r, extra_rounds=extra.value, far_residual=resid.value, safe_clamped=clamped.value)


def fast_sdf(tris, h, mn, mx, fsm_mode=1, gwn_mode=1, threads=None, skip_verify=False, max_conv_rounds=100000,
             signed_parity=False, skip_eikonal=False, lazy_winding=False):
    """The whole fast path (RAST:796-1159). Returns (status, dist or None, sign, stats dict).
    ``signed_parity``: signed crossings in stage [B] (the engine's exact-signs modes).
    ``skip_eikonal``: signs, statuses and statistics only -- no stage [D], which changes no
    voxel the surface tolerance reads; ``dist`` is then the signed band field.
    ``lazy_winding``: the voxels of columns through holes ([C]) and of patch boxes are
    marked (sign 3: the winding number decides) instead of summed; statuses and statistics
    (bar fp64_rechecks) are unchanged, since a probe never reads an undecided voxel and
    makes the fixup's own decision where it would."""
    t, T = _tris(tris)
    mn, mx = _ivec(mn), _ivec(mx)
    dims = mx.astype(np.int64) - mn + 1
    N = int(np.prod(dims)) if (dims > 0).all() else 0
    dist = np.empty(max(N, 1), np.float32)
    sign = np.empty(max(N, 1), np.uint8)
    prm = FastParams(fsm_mode, gwn_mode, threads or default_threads(), max_conv_rounds, 1 if skip_verify else 0,
                     1 if signed_parity else 0, 1 if skip_eikonal else 0, 1 if lazy_winding else 0)
    st = FastStats()
    s = lib().orc_fast_sdf(_p(t), C.c_int(T), C.c_float(h), _p(mn), _p(mx), C.byref(prm), _p(dist), _p(sign),
                           C.byref(st))
    return s, (dist[:N] if s == OK else None), sign[:N], st.as_dict()


def legacy_sdf(tris, h, mn, mx, gwn_mode=1, threads=None):
    """Legacy exact kernel mesh_to_sdf_kernel (RAST:97-185)."""
    t, T = _tris(tris)
    mn, mx = _ivec(mn), _ivec(mx)
    N = int(np.prod(mx.astype(np.int64) - mn + 1))
    out = np.empty(N, np.float32)
    lib().orc_legacy_sdf(_p(t), C.c_int(T), C.c_float(h), _p(mn), _p(mx), C.c_int(gwn_mode), _p(out),
                         C.c_int(threads or default_threads()))
    return out


def lattice(verts, h):
    """build_from_mesh lattice (RAST:1354-1372)."""
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    mn = np.zeros(3, np.int32)
    mx = np.zeros(3, np.int32)
    lib().orc_lattice(_p(v), C.c_longlong(len(v)), C.c_float(h), _p(mn), _p(mx))
    return mn, mx


def build_triangles(verts, faces):
    """Deterministic gpu_build_cuda_triangles_kernel (RAST:1321-1337, MATH:484-514)."""
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
    out = np.empty((len(f), 12), np.float32)
    k = lib().orc_build_triangles(_p(v), C.c_longlong(len(v)), _p(f), C.c_longlong(len(f)), _p(out))
    return out[:k]


# ---- the reference's own primitives (oracle/_ref), where available ------------------
def ref_lib():
    if not REF_LIB_PATH.exists():
        return None
    L = C.CDLL(str(REF_LIB_PATH))
    return L


def parse_binary_stl(data: bytes):
    """Binary STL decode + weld (cuda_mesh_io.cu:524-722). Returns (status, vertices (V,3),
    indices (I,), normals (T,3))."""
    b = np.frombuffer(data, np.uint8)
    T = int(np.frombuffer(data[80:84], np.uint32)[0]) if len(data) >= 84 else 0
    verts = np.zeros((max(3 * T, 1), 3), np.float32)
    idx = np.zeros(max(3 * T, 1), np.uint32)
    normals = np.zeros((max(T, 1), 3), np.float32)
    nv, ni = C.c_int64(0), C.c_int64(0)
    L = lib()
    L.orc_parse_binary_stl.restype = C.c_int
    st = L.orc_parse_binary_stl(_p(b), C.c_size_t(len(data)), _p(verts), _p(idx), _p(normals), C.byref(nv),
                                C.byref(ni))
    return st, verts[:nv.value], idx[:ni.value], normals[:T]


def parse_obj(text: bytes):
    """ASCII OBJ decode (cuda_mesh_io.cu:859-1090). Returns (status, vertices (V,3), indices (I,))."""
    n = len(text)
    cap = n // 10 + 1024
    buf = np.frombuffer(text, np.uint8)
    verts = np.zeros((cap, 3), np.float32)
    idx = np.zeros(cap * 6, np.uint32)
    nv, ni = C.c_int64(0), C.c_int64(0)
    L = lib()
    L.orc_parse_obj.restype = C.c_int
    st = L.orc_parse_obj(_p(buf), C.c_size_t(n), _p(verts), _p(idx), C.byref(nv), C.byref(ni))
    return st, verts[:nv.value], idx[:ni.value]


def parse_ascii_stl(text: bytes):
    """ASCII STL decode (cuda_mesh_io.cu:1094-1325). Returns (status, vertices (V,3), indices (I,))."""
    n = len(text)
    L = lib()
    L.orc_ascii_stl_capacity.restype = C.c_int64
    cap = int(L.orc_ascii_stl_capacity(C.c_size_t(n)))
    buf = np.frombuffer(text, np.uint8) if n else np.zeros(1, np.uint8)
    verts = np.zeros((cap, 3), np.float32)
    idx = np.zeros(cap, np.uint32)
    nv, ni = C.c_int64(0), C.c_int64(0)
    L.orc_parse_ascii_stl.restype = C.c_int
    st = L.orc_parse_ascii_stl(_p(buf), C.c_size_t(n), _p(verts), _p(idx), C.byref(nv), C.byref(ni))
    return st, verts[:nv.value], idx[:ni.value]


def extract_iso_surface(grid, dims, voxel_size, origin, iso, table):
    """Marching cubes (cuda_marching_cubes.cu:829-951) with the edge table `table`
    (256 x 16 int8). Returns (vertices (V,3), indices (I,))."""
    g = np.ascontiguousarray(grid, np.float32).ravel()
    d = np.asarray(dims, np.int32)
    o = np.asarray(origin, np.float32)
    t = np.ascontiguousarray(table, np.int8).ravel()
    nv, ni = C.c_int64(0), C.c_int64(0)
    L = lib()
    L.orc_extract_iso_surface.restype = C.c_int
    L.orc_extract_iso_surface(_p(g), _p(d), C.c_float(voxel_size), _p(o), C.c_float(iso), _p(t), None, None,
                              C.byref(nv), C.byref(ni))
    verts = np.zeros((max(nv.value, 1), 3), np.float32)
    idx = np.zeros(max(ni.value, 1), np.uint32)
    L.orc_extract_iso_surface(_p(g), _p(d), C.c_float(voxel_size), _p(o), C.c_float(iso), _p(t), _p(verts), _p(idx),
                              C.byref(nv), C.byref(ni))
    return verts[:nv.value], idx[:ni.value]


def interior_volume(grid, voxel_size):
    """compute_sdf_interior_volume_gpu (cuda_viewport_gl.cu:702-741, kernel :84-112):
    (float32(count) * float32(h h h), count) over the voxels with value <= 0."""
    g = np.asarray(grid, np.float32).ravel()
    c = int(np.count_nonzero(g <= np.float32(0)))
    h = np.float32(voxel_size)
    return np.float32(np.float32(c) * np.float32(np.float32(h * h) * h)), c


def find_default_seed(grid, dims, min_coord, voxel_size, min_p, max_p, desired_margin):
    """find_default_seed_gpu (cuda_viewport_packers.cu:304-384, kernel :235-276), float32
    step by step: grid minimum (values below 1e30), margin, score 10 z_height + 0.5 xy
    distance, lowest (score, index)."""
    F = np.float32
    g = np.asarray(grid, np.float32).ravel()
    h = F(voxel_size)
    mnp, mxp = np.asarray(min_p, np.float32), np.asarray(max_p, np.float32)
    cx, cy = F((mnp[0] + mxp[0]) * F(0.5)), F((mnp[1] + mxp[1]) * F(0.5))
    seed = np.array([cx, cy, F(mnp[2] + F(F(2.0) * h))], np.float32)
    finite = g[g < F(1e30)]
    m = F(finite.min()) if finite.size else F(1e30)
    margin = F(max(F(desired_margin), F(m * F(0.65)))) if m < 0 else F(m + h)
    idx = np.nonzero(g <= margin)[0]
    if idx.size == 0:
        return seed
    dx, dy = int(dims[0]), int(dims[1])
    x, y, z = idx % dx, (idx // dx) % dy, idx // (dx * dy)
    px = ((np.asarray(min_coord[0]) + x).astype(np.float32) * h).astype(np.float32)
    py = ((np.asarray(min_coord[1]) + y).astype(np.float32) * h).astype(np.float32)
    pz = ((np.asarray(min_coord[2]) + z).astype(np.float32) * h).astype(np.float32)
    ex, ey = (px - cx).astype(np.float32), (py - cy).astype(np.float32)
    xy = np.sqrt((ex * ex).astype(np.float32) + (ey * ey).astype(np.float32)).astype(np.float32)
    zh = np.maximum(F(0), (pz - mnp[2]).astype(np.float32))
    score = ((zh * F(10)).astype(np.float32) + (xy * F(0.5)).astype(np.float32)).astype(np.float32)
    u = score.view(np.uint32)
    key = np.where(u & 0x80000000, ~u, u | 0x80000000).astype(np.uint64) << np.uint64(32)
    key |= (idx.astype(np.uint64) & np.uint64(0xffffffff))
    b = int(idx[np.argmin(key)])
    x, y, z = b % dx, (b // dx) % dy, b // (dx * dy)
    return np.array([F(F(min_coord[0] + x) * h), F(F(min_coord[1] + y) * h), F(F(min_coord[2] + z) * h)], np.float32)


def orient_mesh(vertices, indices):
    """Orientation pre-pass (cuda_mesh_topology.cu:707-842). Returns (indices oriented,
    orientable, had_inconsistent_winding, was_inverted, signed volume)."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices, np.uint32).ravel().copy()
    o, i, w = C.c_int32(0), C.c_int32(0), C.c_int32(0)
    vol = C.c_double(0.0)
    L = lib()
    L.orc_orient_mesh.restype = C.c_int
    L.orc_orient_mesh(_p(v), C.c_int64(len(v)), _p(idx), C.c_int64(len(idx)), C.byref(o), C.byref(i), C.byref(w),
                      C.byref(vol))
    return idx, bool(o.value), bool(i.value), bool(w.value), vol.value
