"""GPU iso-surface extraction (csrc/k_iso.cu) through the C ABI against the oracle's
marching cubes with the same generated table: vertices and indices bit for bit, on random
grids (every case and ambiguous face), a sphere's distance field, and the engine's own
device-resident SDF output read in place (no upload)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _table(engine):
    from gbsdf import _lib

    t = np.zeros((256, 16), np.int8)
    assert _lib.load().gbsdf_iso_surface_table(t.ctypes.data) == 0
    return t


def _check(engine, oracle, grid, dims, h, origin, iso, table):
    gv, gi = engine.extract_iso_surface(grid, dims, h, origin, iso)
    ov, oi = oracle.extract_iso_surface(grid, dims, h, origin, iso, table)
    assert len(oi) > 0
    assert np.array_equal(gv.view(np.uint32), ov.view(np.uint32))
    assert np.array_equal(gi, oi)
    return gv, gi


def test_random_and_sphere_grids(engine, oracle):
    table = _table(engine)
    rng = np.random.default_rng(1)
    for dims in ((9, 7, 5), (33, 17, 20), (64, 40, 31)):
        g = rng.normal(0, 1, dims[::-1]).astype(np.float32)
        g[rng.random(g.shape) < 0.05] = 0.0
        _check(engine, oracle, g, dims, 0.25, (-1.5, 2.0, 0.125), 0.0, table)
        _check(engine, oracle, g, dims, 0.25, (0.0, 0.0, 0.0), 0.3, table)
        gn = g.copy()
        gn[rng.random(g.shape) < 0.03] = np.nan  # NaN corners: outside, midpoint vertices
        _check(engine, oracle, gn, dims, 0.25, (0.0, 0.0, 0.0), 0.0, table)
    n, h = 96, 0.05
    ax = (np.arange(n) - n / 2) * h
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    g = (np.sqrt(x * x + y * y + z * z) - 1.7).astype(np.float32)
    v, i = _check(engine, oracle, g, (n, n, n), h, (ax[0], ax[0], ax[0]), 0.0, table)
    assert np.abs(np.linalg.norm(v, axis=1) - 1.7).max() < 0.05 * h


def test_device_resident_sdf(engine, oracle):
    """The SDF stays on the device: extraction reads the engine's output tensor in place and
    equals extraction from a host copy, and the oracle."""
    import torch

    from gbsdf import meshgen

    v, f = meshgen.mug(segments=64, n_bottom=3, n_wall=6, n_rim=1, handle_path=16, handle_around=12)
    mn, mx = engine.mesh_lattice(v.astype(np.float32), 1.5)
    dims = (mx - mn + 1).astype(np.int64)
    out = torch.empty(int(np.prod(dims)), dtype=torch.float32, device="cuda")
    grid, mn2, mx2, _ = engine.build_from_mesh(v.astype(np.float32), f.astype(np.uint32).ravel(), 1.5, out=out)
    origin = mn.astype(np.float32) * np.float32(1.5)
    dv, di = engine.extract_iso_surface(out, dims, 1.5, origin, 0.0)
    host = out.cpu().numpy()
    hv, hi = engine.extract_iso_surface(host, dims, 1.5, origin, 0.0)
    assert np.array_equal(dv.view(np.uint32), hv.view(np.uint32)) and np.array_equal(di, hi)
    ov, oi = oracle.extract_iso_surface(host, dims, 1.5, origin, 0.0, _table(engine))
    assert np.array_equal(dv.view(np.uint32), ov.view(np.uint32)) and np.array_equal(di, oi)
    # outputs on the device too
    tv, ti = engine.extract_iso_surface(out, dims, 1.5, origin, 0.0, outputs_on_device=True)
    assert np.array_equal(tv.cpu().numpy().view(np.uint32), dv.view(np.uint32))
    assert np.array_equal(ti.cpu().numpy().view(np.uint32), di)
    # a closed, outward surface of the mug
    tri = di.reshape(-1, 3)
    a, b, c = (dv[tri[:, k]].astype(np.float64) for k in range(3))
    assert np.einsum("ij,ij->i", a, np.cross(b, c)).sum() > 0


def test_iso_surface_edges(engine):
    e = engine.extract_iso_surface(np.zeros(8, np.float32), (8, 1, 1), 1.0, (0, 0, 0))
    assert len(e[0]) == 0 and len(e[1]) == 0  # no cube: empty mesh
    e = engine.extract_iso_surface(np.ones(27, np.float32), (3, 3, 3), 1.0, (0, 0, 0))
    assert len(e[1]) == 0  # nothing inside
    with pytest.raises(engine.GbsdfError):
        engine.extract_iso_surface(np.zeros(8, np.float32), (2, 2, 2), 0.0, (0, 0, 0))  # bad voxel size


def test_volume_and_seed(engine, oracle):
    """gbsdf_interior_volume / gbsdf_find_default_seed against the oracle, host and device
    grids, on a sphere's field and on the engine's own mug SDF."""
    import torch

    from gbsdf import meshgen

    rng = np.random.default_rng(5)
    n, h = 70, 0.1
    ax = (np.arange(n) - 35) * h
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    g = (np.sqrt(x * x + y * y + (z - 0.3) ** 2) - 2.5).astype(np.float32)
    v, f = meshgen.mug(segments=48, n_bottom=3, n_wall=5, n_rim=1, handle_path=12, handle_around=10)
    out, mn, mx, _ = engine.build_from_mesh(v.astype(np.float32), f.astype(np.uint32).ravel(), 1.5)
    cases = [(g, (n, n, n), (-35, -35, -35), h, (-3.0, -2.5, -2.0), (3.0, 3.5, 2.0), -0.4),
             (g + rng.normal(0, 1e-3, g.shape).astype(np.float32), (n, n, n), (-35, -35, -35), h, (-3, -3, -3),
              (3, 3, 3), -9.0),
             (out, mx - mn + 1, mn, 1.5, v.min(0), v.max(0), -4.0)]
    for grid, dims, mc, hh, lo, hi, margin in cases:
        for dev in (False, True):
            gg = torch.from_numpy(grid).cuda() if dev else grid
            vol, cnt = engine.interior_volume(gg, hh)
            ovol, ocnt = oracle.interior_volume(grid, hh)
            assert cnt == ocnt and vol == ovol
            s = engine.find_default_seed(gg, dims, mc, hh, lo, hi, margin)
            os_ = oracle.find_default_seed(grid, dims, mc, hh, lo, hi, margin)
            assert np.array_equal(s, os_), (s, os_)
