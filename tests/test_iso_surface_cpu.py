"""The iso-surface triangle table (gbsdf_iso_surface_table, generated in the library, no
GPU needed) and the oracle's marching cubes (oracle/meshio_oracle.cpp, the restatement of
cuda_marching_cubes.cu:829-951 the GPU kernels are compared with):
* every case's triangles use exactly its crossing edges (each at least once) and face
  outward -- from the corners at or below iso towards those above;
* on grids of random values (every case and every ambiguous face occurs) the extracted
  surface is closed: every mesh edge is shared by exactly two triangles, with opposite
  directions (consistently oriented), thanks to the sealed border;
* the surface of a sphere's distance field has Euler characteristic 2 and its vertices
  lie within the interpolation error of the sphere."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

CORNER = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)], float)
EDGE = [(0, 1), (1, 2), (3, 2), (0, 3), (4, 5), (5, 6), (7, 6), (4, 7), (0, 4), (1, 5), (2, 6), (3, 7)]


@pytest.fixture(scope="module")
def table():
    import __graft_entry__

    __graft_entry__.build()
    from gbsdf import _lib

    t = np.zeros((256, 16), np.int8)
    assert _lib.load().gbsdf_iso_surface_table(t.ctypes.data) == 0
    return t


def test_table_cases(table):
    for cs in range(256):
        ins = [(cs >> i) & 1 for i in range(8)]
        crossing = {e for e, (a, b) in enumerate(EDGE) if ins[a] != ins[b]}
        row = table[cs]
        n = 0
        while n < 5 and row[3 * n] >= 0:
            n += 1
        assert (row[3 * n:] == -1).all(), cs
        used = set(int(e) for e in row[:3 * n])
        assert used == crossing, cs
        total = 0.0
        for t in range(n):  # no triangle faces inward; the case's area vector faces outward
            p = [(CORNER[EDGE[e][0]] + CORNER[EDGE[e][1]]) / 2 for e in row[3 * t:3 * t + 3]]
            nrm = np.cross(p[1] - p[0], p[2] - p[0])
            g = sum(CORNER[b] - CORNER[a] if ins[a] else CORNER[a] - CORNER[b]
                    for e in row[3 * t:3 * t + 3] for a, b in [EDGE[e]])
            assert nrm @ g >= 0, cs
            total += nrm @ g
        assert n == 0 or total > 0, cs


def _closed(idx):
    tri = idx.reshape(-1, 3).astype(np.int64)
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
    key = e[:, 0] * (1 << 32) + e[:, 1]
    rev = e[:, 1] * (1 << 32) + e[:, 0]
    u, c = np.unique(key, return_counts=True)
    assert (c == 1).all()  # no directed edge twice: consistent orientation
    assert np.isin(rev, key).all()  # every edge has its opposite: closed


def test_random_grids_closed(table):
    rng = np.random.default_rng(0)
    for dims in ((7, 6, 5), (12, 9, 11), (9, 9, 9), (16, 5, 7), (6, 13, 8), (10, 10, 10)):
        g = rng.normal(0, 1, dims[::-1]).astype(np.float32)
        g[rng.random(g.shape) < 0.1] = 0.0  # values exactly at iso (inside)
        v, i = O.extract_iso_surface(g, dims, 0.5, (0.0, 0.0, 0.0), 0.0, table)
        assert len(i) % 3 == 0 and len(i) > 0
        _closed(i)
        assert i.max() < len(v)


def test_sphere_surface(table):
    n, h, r = 40, 0.1, 1.3
    ax = (np.arange(n) - n / 2 + 0.5) * h
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    g = (np.sqrt(x * x + y * y + z * z) - r).astype(np.float32)
    origin = (ax[0], ax[0], ax[0])
    v, i = O.extract_iso_surface(g, (n, n, n), h, origin, 0.0, table)
    _closed(i)
    tri = i.reshape(-1, 3)
    edges = {tuple(sorted(e)) for t in tri for e in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0]))}
    assert len(v) - len(edges) + len(tri) == 2
    assert np.abs(np.linalg.norm(v, axis=1) - r).max() < 0.05 * h  # linear interpolation of |p| - r
    # outward: the signed volume is positive
    a, b, c = v[tri[:, 0]].astype(np.float64), v[tri[:, 1]].astype(np.float64), v[tri[:, 2]].astype(np.float64)
    assert np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6 > 0


def test_volume_and_seed_oracle():
    """Interior volume and default seed (the other consumers of the SDF) on a sphere's
    distance field: the volume of the voxels inside, the seed at the bottom of the ball shrunk
    by the margin, on the vertical through the box centre."""
    n, h, r = 60, 0.1, 2.2
    ax = (np.arange(n) - 30) * h  # lattice points (min + i) h, min = -30
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    g = (np.sqrt(x * x + y * y + z * z) - r).astype(np.float32)
    vol, cnt = O.interior_volume(g, h)
    assert cnt == int((g <= 0).sum()) and abs(vol - 4 / 3 * np.pi * r ** 3) < 0.02 * 4 / 3 * np.pi * r ** 3
    seed = O.find_default_seed(g, (n, n, n), (-30, -30, -30), h, (-3.0, -3.0, -3.0), (3.0, 3.0, 3.0), -0.5)
    assert abs(seed[0]) < 1e-6 and abs(seed[1]) < 1e-6
    assert -r + 0.5 - h <= seed[2] <= -r + 0.5 + h  # lowest voxel with value <= -0.5
    # nothing inside: the margin becomes min + h, the seed is still the lowest central voxel
    seed = O.find_default_seed(g + np.float32(10), (n, n, n), (-30, -30, -30), h, (-3.0, -3.0, -3.0),
                               (3.0, 3.0, 3.0), -0.5)
    assert abs(seed[0]) < 1e-6 and abs(seed[1]) < 1e-6
