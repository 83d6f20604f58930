"""Generate golden vectors for the geometry primitives from the reference's OWN code.

Runs only where the reference tree exists: it compiles
native/src/core/math_utils.cuh (point_triangle_distance_sq, MATH:43-106;
triangle_solid_angle, MATH:109-132) with a glm stand-in into oracle/_ref (see
oracle/build_ref.sh), evaluates both primitives on seeded inputs that cover every
Voronoi region, near-degenerate triangles and points within 1e-6 of a vertex, and
writes tests/golden/primitives.npz. The oracle's restatement must reproduce these
values bit for bit (tests/test_oracle_golden.py).

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402


def inputs(seed=20261203, n=6000):
    rng = np.random.default_rng(seed)
    tris = rng.normal(0, 3.0, size=(n, 9)).astype(np.float32)
    pts = rng.normal(0, 4.0, size=(n, 3)).astype(np.float32)
    k = n // 6
    # points at / near vertices (solid-angle cut-off 1e-6, vertex regions)
    pts[:k] = tris[:k, 0:3] + rng.normal(0, 1e-7, size=(k, 3)).astype(np.float32)
    # points near edges and faces
    w = rng.dirichlet([1, 1, 1], size=k).astype(np.float32)
    face = w[:, :1] * tris[k:2 * k, 0:3] + w[:, 1:2] * tris[k:2 * k, 3:6] + w[:, 2:3] * tris[k:2 * k, 6:9]
    pts[k:2 * k] = face + rng.normal(0, 1e-3, size=(k, 3)).astype(np.float32)
    t = rng.random((k, 1)).astype(np.float32)
    edge = (1 - t) * tris[2 * k:3 * k, 0:3] + t * tris[2 * k:3 * k, 3:6]
    pts[2 * k:3 * k] = edge + rng.normal(0, 1e-2, size=(k, 3)).astype(np.float32)
    # near-degenerate (sliver) triangles
    tris[3 * k:4 * k, 6:9] = tris[3 * k:4 * k, 0:3] + 1e-4 * (tris[3 * k:4 * k, 3:6] - tris[3 * k:4 * k, 0:3])
    # large lattice-scale coordinates (0.1 mm voxels, grids of ~1000)
    tris[4 * k:5 * k] *= 20.0
    pts[4 * k:5 * k] *= 20.0
    return np.ascontiguousarray(pts), np.ascontiguousarray(tris)


def main():
    lib_path = O.build_ref()
    if lib_path is None:
        raise SystemExit("reference tree not present; golden vectors cannot be regenerated here")
    L = C.CDLL(str(lib_path))
    pts, tris = inputs()
    n = len(pts)
    d2 = np.empty(n, np.float32)
    om = np.empty(n, np.float32)
    L.ref_ptd_batch(pts.ctypes.data_as(C.c_void_p), tris.ctypes.data_as(C.c_void_p), C.c_longlong(n),
                    d2.ctypes.data_as(C.c_void_p))
    L.ref_solid_angle_batch(pts.ctypes.data_as(C.c_void_p), tris.ctypes.data_as(C.c_void_p), C.c_longlong(n),
                            om.ctypes.data_as(C.c_void_p))
    out = Path(__file__).resolve().parent / "primitives.npz"
    np.savez_compressed(out, pts=pts, tris=tris, d2=d2, omega=om)
    print(f"wrote {out}: {n} cases")


if __name__ == "__main__":
    main()
