"""The oracle is pinned before it is trusted (CPU only).

* Geometry primitives: bit-exact against golden vectors produced by the reference's
  own point_triangle_distance_sq / triangle_solid_angle (math_utils.cuh:43-132),
  compiled from the reference tree (tests/golden/make_golden.py).
* Known answers the reference's verification suite uses: analytical sphere SDF
  (cuda_verification.cu:511-531, max error < 1.5 mm on a 37^3 grid at 1 mm) and the
  dirty-mesh winding classification thresholds (harness_vessel_tests.cpp:54-121,
  cuda_verification.cu:266-281).
* The eikonal update: hand-checked values, and the non-monotonicity of the reference
  update that makes its fixed point schedule-dependent.
"""
import math
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "primitives.npz"


def test_primitives_bit_exact_against_reference_code(oracle):
    z = np.load(GOLD)
    d2 = oracle.ptd_batch(z["pts"], z["tris"])
    om = oracle.solid_angle_batch(z["pts"], z["tris"])
    assert np.array_equal(d2.view(np.uint32), z["d2"].view(np.uint32))
    assert np.array_equal(om.view(np.uint32), z["omega"].view(np.uint32))


def test_golden_covers_cutoff_and_regions():
    z = np.load(GOLD)
    assert (z["omega"] == 0).sum() > 500  # vertex cut-off |v - p| <= 1e-6
    assert np.isfinite(z["d2"]).all() and (z["d2"] >= 0).all()


def test_solid_angle_octant(oracle):
    # right octant triangle seen from the origin: -pi/2 ... the reference probe printed -pi
    p = np.zeros((1, 3), np.float32)
    t = np.array([[1, 0, 0, 0, 0, 1, 0, 1, 0]], np.float32)
    om = oracle.solid_angle_batch(p, t)[0]
    assert abs(abs(om) - math.pi / 2) < 1e-5


def test_godunov_reference_values(oracle):
    h = 1.0
    assert oracle.godunov(0.0, 1e30, 1e30, h) == pytest.approx(1.0)          # 1D
    assert oracle.godunov(0.0, 0.0, 1e30, h) == pytest.approx(math.sqrt(2) / 2)  # 2D symmetric
    assert oracle.godunov(0.0, 0.0, 0.0, h) == pytest.approx(1 / math.sqrt(3))  # 3D symmetric


def test_reference_update_is_not_monotone(oracle):
    # RAST:418 halves the pairwise sum of the 3D discriminant; raising one neighbour can
    # lower the update across the 2D->3D switch. The corrected update is monotone.
    h = 1.0
    rng = np.random.default_rng(1)
    ref_viol = 0
    for _ in range(20000):
        a, b, c = np.sort(rng.random(3) * 1.5).astype(np.float32)
        dc = np.float32(rng.random() * 0.2)
        lo = oracle.godunov(a, b, c, h)
        hi = oracle.godunov(a, b, c + dc, h)
        ref_viol += hi < lo - 1e-6
    assert ref_viol > 0
    L = oracle.lib()
    import ctypes as C

    L.orc_godunov_exact.restype = C.c_float
    L.orc_godunov_exact.argtypes = [C.c_float] * 4
    viol = 0
    for _ in range(20000):
        a, b, c = np.sort(rng.random(3) * 1.5).astype(np.float32)
        dc = np.float32(rng.random() * 0.2)
        viol += L.orc_godunov_exact(a, b, c + dc, h) < L.orc_godunov_exact(a, b, c, h) - 1e-6
    assert viol == 0


def _sphere(r, nlat=32, nlon=32):
    th = np.linspace(0, np.pi, nlat + 1)[1:-1]
    ph = np.arange(nlon) * 2 * np.pi / nlon
    T, P = np.meshgrid(th, ph, indexing="ij")
    v = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
    v = np.vstack([v, [[0, 0, 1], [0, 0, -1]]]) * r
    R, A = nlat - 1, nlon
    f = []
    for i in range(R - 1):
        for j in range(A):
            a, b, c, d = i * A + j, i * A + (j + 1) % A, (i + 1) * A + (j + 1) % A, (i + 1) * A + j
            f += [(a, c, b), (a, d, c)]
    for j in range(A):
        f.append((R * A, j, (j + 1) % A))
        f.append((R * A + 1, (R - 1) * A + (j + 1) % A, (R - 1) * A + j))
    return v.astype(np.float32), np.asarray(f, np.int64)


def test_legacy_sphere_known_answer(oracle):
    # cuda_verification.cu:1076-1095 / :511-531: sphere R=15 on [-18,18]^3 at 1 mm, error < 1.5 mm
    from gbsdf import meshgen

    v, f = _sphere(15.0)
    if meshgen.signed_volume(v, f) < 0:
        f = f[:, [0, 2, 1]]
    tris = meshgen.to_triangles(v, f)
    out = oracle.legacy_sdf(tris, 1.0, (-18, -18, -18), (18, 18, 18), gwn_mode=1)
    g = np.arange(-18, 19, dtype=np.float32)
    Z, Y, X = np.meshgrid(g, g, g, indexing="ij")
    ana = np.sqrt(X * X + Y * Y + Z * Z) - 15.0
    assert np.max(np.abs(out - ana.ravel())) < 1.5


def _hash01(x):
    # dev_hash_01 (math_utils.cuh:219-226), vectorised over uint32
    x = np.asarray(x, np.uint64) & 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return (x & 0x00FFFFFF).astype(np.float64) / 16777216.0


def _open_box():
    v = np.array([[-10, -10, -10], [10, -10, -10], [10, 10, -10], [-10, 10, -10],
                  [-10, -10, 10], [10, -10, 10], [10, 10, 10], [-10, 10, 10]], np.float32)
    f = np.array([0, 2, 1, 0, 3, 2, 0, 1, 5, 0, 5, 4, 1, 2, 6, 1, 6, 5, 2, 3, 7, 2, 7, 6, 3, 0, 4, 3, 4, 7]).reshape(-1, 3)
    return v, f


def test_dirty_mesh_gwn_open_box(oracle):
    # harness_vessel_tests.cpp:58-75 + cuda_verification.cu:209-233 (mode 0) and :266-281:
    # >= 99% of 10,000 hash-seeded points classified with in >= 0.45, out < 0.35.
    from gbsdf import meshgen

    v, f = _open_box()
    tris = meshgen.to_triangles(v, f)
    seed = 42
    i = np.arange(10000, dtype=np.uint64)
    s0 = (seed + i * 9973 + 17) & 0xFFFFFFFF
    pts = np.zeros((10000, 3))
    inn = i < 5000
    pts[inn, 0] = -8.5 + 17.0 * _hash01(s0[inn] + 1)
    pts[inn, 1] = -8.5 + 17.0 * _hash01(s0[inn] + 2)
    pts[inn, 2] = -8.5 + 11.5 * _hash01(s0[inn] + 3)
    for k in np.nonzero(~inn)[0]:
        pts[k] = (25, 25, 25)
        for att in range(64):
            x = -35 + 70 * _hash01(s0[k] + att * 3 + 1)
            y = -35 + 70 * _hash01(s0[k] + att * 3 + 2)
            z = -35 + 70 * _hash01(s0[k] + att * 3 + 3)
            if not (abs(x) <= 12 and abs(y) <= 12 and -12 <= z <= 12):
                pts[k] = (x, y, z)
                break
    w = oracle.gwn_points_f64(tris, pts.astype(np.float32))
    ok = np.where(inn, w >= 0.45, w < 0.35)
    assert ok.mean() >= 0.99


def _gwn_points(mode, seed):
    """gpu_generate_gwn_test_points_kernel (cuda_verification.cu:209-263), modes 1 and 2."""
    i = np.arange(10000, dtype=np.uint64)
    s0 = (seed + i * 9973 + 17) & 0xFFFFFFFF
    inn = i < 5000
    pts = np.zeros((10000, 3))
    if mode == 1:
        r = np.where(inn, 13.5 * _hash01(s0 + 1), 16.5 + 18.5 * _hash01(s0 + 1))
        u = -1.0 + 2.0 * _hash01(s0 + 2)
        th = 2 * np.pi * _hash01(s0 + 3)
        sq = np.sqrt(np.maximum(0.0, 1.0 - u * u))
        pts = r[:, None] * np.stack([sq * np.cos(th), sq * np.sin(th), u], -1)
        return pts, inn
    pts[inn, 0] = -8.5 + 25.0 * _hash01(s0[inn] + 1)
    pts[inn, 1] = -8.5 + 17.0 * _hash01(s0[inn] + 2)
    pts[inn, 2] = -8.5 + 17.0 * _hash01(s0[inn] + 3)
    for k in np.nonzero(~inn)[0]:
        pts[k] = (28, 28, 28)
        for att in range(64):
            x = -35 + 70 * _hash01(s0[k] + att * 3 + 1)
            y = -35 + 70 * _hash01(s0[k] + att * 3 + 2)
            z = -35 + 70 * _hash01(s0[k] + att * 3 + 3)
            if not (-12 <= x <= 20 and abs(y) <= 12 and abs(z) <= 12):
                pts[k] = (x, y, z)
                break
    return pts, inn


def test_dirty_mesh_gwn_inverted_sphere(oracle):
    # harness_vessel_tests.cpp:77-83 + cuda_verification.cu:236-243, :266-281: a sphere
    # (R 15, 48 x 48) with every winding flipped, oriented back by the orientation pre-pass;
    # >= 99% of 10,000 points classified with in >= 0.50, out < 0.25
    from gbsdf import meshgen

    v, f = _sphere(15.0, 48, 48)
    if meshgen.signed_volume(v, f) < 0:
        f = f[:, [0, 2, 1]]
    idx, orientable, inconsistent, inverted, vol = oracle.orient_mesh(v, f[:, [0, 2, 1]].astype(np.uint32))
    assert orientable and inverted and vol > 0
    pts, inn = _gwn_points(1, 1337)
    w = oracle.gwn_points_f64(meshgen.to_triangles(v, idx.reshape(-1, 3)), pts.astype(np.float32))
    ok = np.where(inn, w >= 0.50, w < 0.25)
    assert ok.mean() >= 0.99


def test_dirty_mesh_gwn_intersecting_cubes(oracle):
    # harness_vessel_tests.cpp:85-102 + cuda_verification.cu:244-262, :266-281: two
    # overlapping closed cubes; >= 99% of 10,000 points classified (in >= 0.45, out < 0.25)
    from gbsdf import meshgen

    c = np.array([[-10, -10, -10], [10, -10, -10], [10, 10, -10], [-10, 10, -10],
                  [-10, -10, 10], [10, -10, 10], [10, 10, 10], [-10, 10, 10]], np.float32)
    v = np.vstack([c, c + np.array([8, 0, 0], np.float32)])
    q = np.array([0, 2, 1, 0, 3, 2, 4, 5, 6, 4, 6, 7, 0, 1, 5, 0, 5, 4,
                  1, 2, 6, 1, 6, 5, 2, 3, 7, 2, 7, 6, 3, 0, 4, 3, 4, 7]).reshape(-1, 3)
    f = np.vstack([q, q + 8])
    pts, inn = _gwn_points(2, 9001)
    w = oracle.gwn_points_f64(meshgen.to_triangles(v, f), pts.astype(np.float32))
    ok = np.where(inn, w >= 0.45, w < 0.25)
    assert ok.mean() >= 0.99


def eikonal_fraction(grid, dims, mn, dx, R, seed=1337, n=55000, tol=0.02):
    """The reference's eikonal property check, case (a) (harness_eikonal_cuda_tests.cpp:
    55-129 with gpu_evaluate_eikonal_field_kernel, cuda_verification.cu:393-505, sample mode
    0): n points on shells R + U(-3 dx, 3 dx) from the hash-seeded directions, the field
    sampled trilinearly (dev_sample_sdf_trilinear, math_utils.cuh:344-389; 1000 outside),
    central differences at dx / 2; returns the fraction with | |grad f| - 1 | <= tol."""
    g = np.asarray(grid, np.float32).reshape(int(dims[2]), int(dims[1]), int(dims[0]))
    i = np.arange(n, dtype=np.uint64)
    s0 = (np.uint64(seed) + i * np.uint64(19997) + np.uint64(31)) & np.uint64(0xFFFFFFFF)
    th = 2 * np.pi * _hash01(s0 + np.uint64(1))
    cp = -1.0 + 2.0 * _hash01(s0 + np.uint64(2))
    sp = np.sqrt(np.maximum(0.0, 1.0 - cp * cp))
    r = R + (-3.0 * dx + 6.0 * dx * _hash01(s0 + np.uint64(3)))
    p = np.stack([r * sp * np.cos(th), r * cp, r * sp * np.sin(th)], -1)
    mn = np.asarray(mn, np.float64)

    def f(q):
        gq = q / dx - mn
        i0 = np.floor(gq).astype(np.int64)
        inside = np.all((i0 >= 0) & (i0 < np.asarray(dims)[None, :] - 1), axis=1)
        i0c = np.clip(i0, 0, np.asarray(dims) - 2)
        fr = gq - i0c
        x0, y0, z0 = i0c[:, 0], i0c[:, 1], i0c[:, 2]
        fx, fy, fz = fr[:, 0], fr[:, 1], fr[:, 2]
        v = lambda a, b, c: g[z0 + c, y0 + b, x0 + a].astype(np.float64)
        c00 = v(0, 0, 0) * (1 - fx) + v(1, 0, 0) * fx
        c10 = v(0, 1, 0) * (1 - fx) + v(1, 1, 0) * fx
        c01 = v(0, 0, 1) * (1 - fx) + v(1, 0, 1) * fx
        c11 = v(0, 1, 1) * (1 - fx) + v(1, 1, 1) * fx
        out = (c00 * (1 - fy) + c10 * fy) * (1 - fz) + (c01 * (1 - fy) + c11 * fy) * fz
        return np.where(inside, out, 1000.0)

    hh = 0.5 * dx
    grad = []
    for k in range(3):
        e = np.zeros(3)
        e[k] = hh
        grad.append((f(p + e) - f(p - e)) / (2 * hh))
    diff = np.abs(np.sqrt(grad[0] ** 2 + grad[1] ** 2 + grad[2] ** 2) - 1.0)
    return float(np.mean(diff <= tol))


def sphere_case(R=20.0, dx=0.35):
    from gbsdf import meshgen

    v, f = _sphere(R, 96, 96)
    if meshgen.signed_volume(v, f) < 0:
        f = f[:, [0, 2, 1]]
    return v.astype(np.float32), f


def test_eikonal_property_sphere(oracle):
    """Harness case (a): sphere R = 20 mm (96 x 96 tessellation) at dx = 0.35 mm on the
    build_from_mesh lattice; the reference passes it when at least 85% of the samples are
    within 0.02 of |grad f| = 1. The oracle's reference-mode build does."""
    from gbsdf import meshgen

    v, f = sphere_case()
    mn, mx = oracle.lattice(v, 0.35)
    st, dist, _, _ = oracle.fast_sdf(meshgen.to_triangles(v, f), 0.35, mn, mx, fsm_mode=0, gwn_mode=1)
    assert st == 0
    frac = eikonal_fraction(dist, mx - mn + 1, mn, 0.35, 20.0)
    assert frac >= 0.85, frac
