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
