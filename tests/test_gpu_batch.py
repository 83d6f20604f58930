"""Batched entry point (gbsdf_compute_mesh_sdf_batch): meshes of uneven size in one call
give the same grids as one call each."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _meshes():
    from gbsdf import meshgen

    out = []
    v, f = meshgen.mug(segments=64, n_bottom=3, n_wall=6, n_rim=1, handle_path=16, handle_around=12)
    vf, mn, mx = meshgen.fit_to_lattice(v, (40, 40, 44), 2.4)
    out.append((meshgen.to_triangles(vf, f), 2.4, mn, mx))
    v, f = meshgen.perturbed_sphere(seed=4, n_lat=24, n_lon=48)
    vf, mn, mx = meshgen.fit_to_lattice(v, (24, 28, 20), 3.0)
    out.append((meshgen.to_triangles(vf, f), 3.0, mn, mx))
    v, f = meshgen.vessel_tree(seed=11, levels=2, around=12, n_len=6, n_cap=2, defects=False)
    vf, mn, mx = meshgen.fit_to_lattice(v, (48, 40, 56), 1.0)
    out.append((meshgen.to_triangles(vf, f), 1.0, mn, mx))
    return out


def test_batch_matches_single_calls(engine):
    meshes = _meshes()
    outs, statuses, stats, _ = engine.compute_mesh_sdf_batch(meshes)
    assert statuses == [0, 0, 0]
    for (tris, h, mn, mx), got, st in zip(meshes, outs, stats):
        ref, res = engine.compute_mesh_sdf(tris, h, mn, mx, path=engine.PATH_FAST)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
        assert st["eikonal_rounds"] == res.stats["eikonal_rounds"]


def test_batch_device_buffers_and_bad_member(engine):
    import torch

    meshes = _meshes()
    bad = (meshes[1][0].copy(), meshes[1][1], meshes[1][2], meshes[1][3])
    bad[0][0, 0] = np.nan
    batch = [(torch.from_numpy(t).cuda(), h, mn, mx) for t, h, mn, mx in [meshes[0], bad, meshes[2]]]
    outs = [torch.full((int(np.prod(mx.astype(np.int64) - mn + 1)),), 5.0, device="cuda") for _, _, mn, mx in batch]
    _, statuses, _, msg = engine.compute_mesh_sdf_batch(batch, outs=outs, raise_on_error=False)
    assert statuses[0] == 0 and statuses[1] == 1 and statuses[2] == 0
    assert "mesh 1" in msg
    assert torch.all(outs[1] == 5.0)
    ref, _ = engine.compute_mesh_sdf(meshes[2][0], *meshes[2][1:], path=engine.PATH_FAST)
    assert np.array_equal(outs[2].cpu().numpy(), ref)


def test_planned_batch_replays_and_follows_new_contents(engine):
    """A planned batch replays its graph: the same contents give the same grids, new
    contents of the same size give the new grids, and contents whose pair lists outgrow
    the plan make the run re-plan itself."""
    meshes = _meshes()
    with engine.Batch(meshes) as b:
        st, stats = b.run()
        assert st == [0, 0, 0]
        first = [o.copy() for o in b.outs]
        st, _ = b.run()
        assert st == [0, 0, 0]
        for a, o in zip(first, b.outs):
            assert np.array_equal(a.view(np.uint32), o.view(np.uint32))
        # new contents in place: shift mesh 0 by a fraction of a voxel, grow mesh 2
        t0, h0, mn0, mx0 = meshes[0]
        t0[:, 0:9] += np.float32(0.37 * h0)
        t2, h2, mn2, mx2 = meshes[2]
        c = t2[:, 0:9].reshape(-1, 3).mean(0)
        v = t2[:, 0:9].reshape(-1, 3)
        t2[:, 0:9] = ((v - c) * np.float32(1.35) + c).reshape(-1, 9)
        st, _ = b.run()
        assert st == [0, 0, 0]
        for (tris, h, mn, mx), got in zip(meshes, b.outs):
            ref, _ = engine.compute_mesh_sdf(tris, h, mn, mx, path=engine.PATH_FAST)
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_planned_batch_exact_signs_and_device_buffers(engine):
    import torch

    meshes = _meshes()
    dev = [(torch.from_numpy(t).cuda(), h, mn, mx) for t, h, mn, mx in meshes]
    outs = [torch.empty(int(np.prod(mx.astype(np.int64) - mn + 1)), device="cuda") for _, _, mn, mx in meshes]
    with engine.Batch(dev, outs=outs, mode=engine.MODE_EXACT_SIGNS) as b:
        st, stats = b.run()
        assert st == [0, 0, 0]
        assert stats[0]["kernel_launches"] > 0
    for (tris, h, mn, mx), got in zip(meshes, outs):
        ref, _ = engine.compute_mesh_sdf(tris, h, mn, mx, mode=engine.MODE_EXACT_SIGNS, path=engine.PATH_FAST)
        assert np.array_equal(got.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_planned_batch_bad_lattice_member(engine):
    meshes = _meshes()
    t, h, mn, mx = meshes[1]
    bad = (t, h, mx, mn)  # max < min: empty lattice
    outs = [np.full(int(np.prod(mx.astype(np.int64) - mn + 1)), 7.0, np.float32) for _, _, mn, mx in meshes]
    with engine.Batch([meshes[0], bad, meshes[2]], outs=outs) as b:
        st, _ = b.run()
    assert st[0] == 0 and st[1] == 1 and st[2] == 0
    assert np.all(outs[1] == 7.0)
